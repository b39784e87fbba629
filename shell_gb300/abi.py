"""ctypes mirrors of the structures of include/shl.h.

Plain Python (no library is loaded here): the CUDA library's binding
(shell_gb300/lib.py) and the CPU oracle, which implements the same header, both
use them.
"""
import ctypes

_d, _i32, _u32 = ctypes.c_double, ctypes.c_int32, ctypes.c_uint32


class ShlMesh(ctypes.Structure):
    _fields_ = [("n_nodes", _u32), ("n_faces", _u32), ("xyz", ctypes.c_void_p), ("faces", ctypes.c_void_p)]


_PARAM_FIELDS = (
    [(n, _d) for n in ("shell_mass_density", "shell_young_modulus", "shell_young_modulus2", "shell_poisson_ratio",
                       "shell_shear_modulus", "bulk_modulus", "memb_stiff_mult", "bend_stiff_mult", "thickness",
                       "damping_alpha", "damping_beta", "damping_gamma", "pressure")]
    + [("pressure_base", _i32), ("pressure_dir", _i32), ("shell_shell_contact", _i32), ("pad0", _i32)]
    + [(n, _d) for n in ("mu_s", "mu_d", "self_damping", "self_friction_damping", "fric_stiff_mult",
                       "friction_stop_velocity", "static_friction_tol", "cell_size_mult", "cell_margin",
                       "neighbor_margin", "dt", "newmark_beta", "newmark_gamma")]
    + [("compat_zero_pressure", _i32), ("precision", _i32), ("stop_on_problem", _i32), ("pad1", _i32)]
    + [("adapt_dt_every", _u32), ("pad2", _i32)]
    + [(n, _d) for n in ("dt_min", "dt_max", "rel_loc_err_min", "rel_loc_err_max")]
    + [("shell_cavity_contact", _i32), ("cavity", _i32)]
    + [(n, _d) for n in ("Rx", "Ry", "Rz", "mu_s_cavity", "mu_d_cavity", "cavity_damping", "cavity_friction_damping")]
)


class ShlParams(ctypes.Structure):
    _fields_ = _PARAM_FIELDS

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in _PARAM_FIELDS if not n.startswith("pad")}


class ShlEnergies(ctypes.Structure):
    _fields_ = [(n, _d) for n in ("Etens", "Ebend", "Eself", "Efric", "Ekin", "area", "volume", "kGauss", "kMean")] + [
        ("Nc", _u32), ("n_pairs", _u32), ("Ecav", _d), ("cavity_force", _d), ("Nc_cav", _u32), ("pad", _u32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class ShlStepReport(ctypes.Structure):
    _fields_ = [("steps_done", _u32), ("worst_problem", _i32), ("time", _d), ("du_sum", _d), ("n_rebuilds", _u32),
                ("rejections", _u32), ("last", ShlEnergies)] + [
        (n, _d) for n in ("sum_dt", "sum_area", "sum_volume", "sum_Nc", "sum_Ekin", "sum_Etens", "sum_Ebend",
                          "sum_Eself", "sum_Efric", "sum_kGauss", "sum_kMean")] + [("stopped", _u32), ("pad", _u32)] + [
        (n, _d) for n in ("sum_pcav", "sum_Nc_cav", "sum_Ecav")]
