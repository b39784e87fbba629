"""ctypes binding of the C ABI in include/shl.h (libshl_gb300.so).

This is the Python side of the drop-in boundary: the structures mirror shl.h
field by field and `Shell` mirrors the ShellSystem methods a host driver calls
(set_parameters/build_cache -> Shell(...), apply_initial_conditions, advance,
save/load state).  The library is loaded from the in-tree build directory; if
it is missing the import fails loudly (there is no fallback implementation).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libshl_gb300.so")

# shl_status
SHL_OK = 0
PROBLEMS = {0: "NO_PROBLEM", 1: "NO_DISP_CHANGE", 2: "LARGE_DISP", 3: "STOP_SIM", 4: "TOO_MANY_CELLS",
            5: "SMALL_TIMESTEP", 6: "CONTACT_PROBLEM", 7: "NOT_FINITE"}
SHL_ERR_ARG, SHL_ERR_CUDA, SHL_ERR_TIMEOUT, SHL_ERR_OOM, SHL_ERR_CAPACITY = 100, 101, 102, 103, 104
CONTACT_LINEAR, CONTACT_SMOOTH, CONTACT_NONE = 0, 1, 2
CS_LOCAL, CS_CARTESIAN, CS_CYLINDRICAL, CS_SPHERICAL = 0, 1, 2, 3
PREC_FP64, PREC_FP32 = 0, 1
ELEMENT_VARIANTS = 14  # SHL_ELEMENT_VARIANTS
CAVITY_BOX, CAVITY_CYLINDER, CAVITY_ELLIPSOID = 0, 1, 2

from shell_gb300.abi import (_PARAM_FIELDS, ShlEnergies, ShlMesh, ShlParams, ShlStepReport,  # noqa: E402,F401
                             _d, _i32, _u32)


_lib = None
RESIDUAL_FP64, RESIDUAL_CORRECT, RESIDUAL_CLEAR, RESIDUAL_CONTACT = 1, 2, 4, 8


def load():
    """Load libshl_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libshl_gb300.so is not built (run `python -m shell_gb300.build`): %s" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    sig = {
        "shl_version": (ctypes.c_char_p, []),
        "shl_last_error": (ctypes.c_char_p, []),
        "shl_status_string": (ctypes.c_char_p, [_i32]),
        "shl_create": (_i32, [ctypes.POINTER(ShlMesh), ctypes.POINTER(ShlParams), ctypes.POINTER(vp)]),
        "shl_destroy": (None, [vp]),
        "shl_apply_initial_conditions": (_i32, [vp, vp, _d, _d]),
        "shl_set_state": (_i32, [vp, vp, vp, vp]),
        "shl_get_state": (_i32, [vp, vp, vp, vp]),
        "shl_set_time": (_i32, [vp, _d, _u32]),
        "shl_get_time": (_i32, [vp, ctypes.POINTER(_d), ctypes.POINTER(_u32)]),
        "shl_eval_forces": (_i32, [vp, vp, vp, _d, vp, vp, ctypes.POINTER(ShlEnergies)]),
        "shl_step": (_i32, [vp, _u32, vp, ctypes.c_int, ctypes.POINTER(ShlStepReport)]),
        "shl_get_contact_pairs": (_i32, [vp, vp, sz, ctypes.POINTER(sz)]),
        "shl_get_contact_state": (_i32, [vp, vp, vp, vp, vp, sz, ctypes.POINTER(sz), ctypes.POINTER(_d)]),
        "shl_set_contact_state": (_i32, [vp, vp, vp, vp, vp, sz, _d]),
        "shl_rebuild_contacts": (_i32, [vp]),
        "shl_get_contact_coords": (_i32, [vp, vp, sz, ctypes.POINTER(sz)]),
        "shl_set_contact_coords": (_i32, [vp, vp, sz]),
        "shl_get_element_fields": (_i32, [vp, vp, vp, vp, vp, vp]),
        "shl_get_mass_damping": (_i32, [vp, vp, vp]),
        "shl_icosphere": (_i32, [_u32, vp, sz, vp, sz, ctypes.POINTER(_u32), ctypes.POINTER(_u32)]),
        "shl_icosphere_off": (_i32, [_u32, vp, sz, ctypes.POINTER(sz)]),
        "shl_read_off": (_i32, [ctypes.c_char_p, vp, sz, vp, sz, ctypes.POINTER(_u32), ctypes.POINTER(_u32)]),
        "shl_gaussian_normal_imperfection": (_i32, [vp, _u32, _d, ctypes.c_uint64, vp]),
        "shl_params_default": (None, [ctypes.POINTER(ShlParams)]),
        "shl_get_stream": (_i32, [vp, ctypes.POINTER(vp)]),
        "shl_upload_pressure_table": (_i32, [vp, vp, _u32]),
        "shl_step_enqueue": (_i32, [vp, _u32]),
        "shl_step_collect": (_i32, [vp, ctypes.POINTER(ShlStepReport)]),
        "shl_time_kernel": (_i32, [vp, ctypes.c_int, ctypes.c_int, sz, ctypes.POINTER(_d)]),
        "shl_measure_fp64_peak": (_i32, [ctypes.POINTER(_d)]),
        "shl_internal_force_noalloc": (_i32, [vp, vp, _d, vp, vp]),
        "shl_profile_step": (_i32, [vp, _d, sz, vp]),
        "shl_batch_create": (_i32, [vp, vp, vp, _u32, ctypes.POINTER(vp)]),
        "shl_batch_layout": (_i32, [vp, ctypes.POINTER(_u32), vp, vp]),
        "shl_batch_contact_stats": (_i32, [vp, vp, vp]),
        "shl_context_size": (_i32, [vp, ctypes.POINTER(_u32), ctypes.POINTER(_u32)]),
        "shl_context_mesh": (_i32, [vp, vp, vp]),
        "shl_get_node_fields": (_i32, [vp, vp, vp, vp, vp, vp]),
        "shl_apply_loaded_state": (_i32, [vp]),
        "shl_save_state_file": (_i32, [vp, ctypes.c_char_p, _u32, _d, _d, vp, _u32]),
        "shl_load_state_file": (_i32, [vp, ctypes.c_char_p, ctypes.POINTER(_u32), ctypes.POINTER(_d),
                                       ctypes.POINTER(_d), vp, _u32, ctypes.POINTER(_u32)]),
        "shl_write_vtu": (_i32, [vp, ctypes.c_char_p]),
        "shl_get_energies": (_i32, [vp, ctypes.POINTER(ShlEnergies)]),
        "shl_mlp_create": (_i32, [vp, _u32, _u32, ctypes.c_uint64, ctypes.POINTER(vp)]),
        "shl_mlp_destroy": (None, [vp]),
        "shl_mlp_set_params": (_i32, [vp, _u32, vp, vp]),
        "shl_mlp_get_params": (_i32, [vp, _u32, vp, vp]),
        "shl_mlp_set_dataset": (_i32, [vp, vp, vp, ctypes.c_uint64]),
        "shl_mlp_train": (_i32, [vp, _u32, _u32, ctypes.c_float, ctypes.c_float, ctypes.c_uint64, vp, _u32]),
        "shl_mlp_predict": (_i32, [vp, vp, _u32, vp]),
        "shl_mlp_gradients": (_i32, [vp, vp, vp, _u32, ctypes.POINTER(_d), vp, vp]),
        "shl_gemm_bf16": (_i32, [vp, vp, _u32, _u32, _u32, vp]),
        "shl_gemm_bf16_time": (_i32, [_u32, _u32, _u32, ctypes.c_int, ctypes.POINTER(_d)]),
        "shl_residual": (_i32, [vp, _d, ctypes.c_int, vp, vp, vp]),
        "shl_set_pressure_function": (_i32, [vp, ctypes.c_char_p]),
        "shl_get_dt": (_i32, [vp, ctypes.POINTER(_d), ctypes.POINTER(_u32)]),
        "shl_set_stop_function": (_i32, [vp, ctypes.c_char_p]),
        "shl_set_cavity_functions": (_i32, [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]),
        "shl_get_cavity_origins": (_i32, [vp, vp]),
        "shl_set_cavity_origins": (_i32, [vp, vp]),
        "shl_scale_damping": (_i32, [vp, _d]),
        "shl_set_element_variant": (_i32, [vp, ctypes.c_int]),
        "shl_get_element_variant": (_i32, [vp, ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, sz, vp]),
        "shl_eval_pressure_function": (_i32, [vp, vp, _u32, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    """Names declared in include/shl.h (for the export check)."""
    return ["shl_version", "shl_last_error", "shl_status_string", "shl_create", "shl_destroy",
            "shl_apply_initial_conditions", "shl_set_state", "shl_get_state", "shl_set_time", "shl_get_time",
            "shl_eval_forces", "shl_step", "shl_get_contact_pairs", "shl_get_contact_state",
            "shl_set_contact_state", "shl_rebuild_contacts", "shl_get_element_fields", "shl_get_mass_damping",
            "shl_icosphere", "shl_icosphere_off", "shl_read_off", "shl_gaussian_normal_imperfection",
            "shl_params_default", "shl_get_stream", "shl_upload_pressure_table", "shl_step_enqueue",
            "shl_step_collect", "shl_time_kernel", "shl_measure_fp64_peak", "shl_internal_force_noalloc",
            "shl_profile_step", "shl_batch_create", "shl_batch_layout", "shl_batch_contact_stats", "shl_context_size",
            "shl_context_mesh",
            "shl_get_node_fields", "shl_apply_loaded_state", "shl_save_state_file", "shl_load_state_file",
            "shl_write_vtu", "shl_get_energies", "shl_mlp_create", "shl_mlp_destroy", "shl_mlp_set_params",
            "shl_mlp_get_params", "shl_mlp_set_dataset", "shl_mlp_train", "shl_mlp_predict", "shl_mlp_gradients",
            "shl_gemm_bf16", "shl_gemm_bf16_time", "shl_residual", "shl_set_pressure_function", "shl_eval_pressure_function",
            "shl_get_dt", "shl_set_stop_function", "shl_set_cavity_functions", "shl_get_cavity_origins",
            "shl_set_cavity_origins", "shl_scale_damping", "shl_set_element_variant", "shl_get_element_variant",
            "shl_get_contact_coords", "shl_set_contact_coords"]


class ShlError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.shl_status_string(status).decode()
        detail = lib.shl_last_error().decode()
        super().__init__("%s: status %d (%s) %s" % (where, status, msg, detail))
        self.status = status


def _ptr(a):
    return None if a is None else a.ctypes.data


def _check(status, where, allow_problem=True):
    if status >= 100 or (status != 0 and not allow_problem):
        raise ShlError(status, where)
    return status


def default_params(**kw):
    lib = load()
    p = ShlParams()
    lib.shl_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def icosphere(level):
    """Closed icosphere mesh (node xyz (V,3) float64, faces (F,3) uint32)."""
    lib = load()
    nv, nf = _u32(), _u32()
    _check(lib.shl_icosphere(level, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nf)), "shl_icosphere")
    X = np.zeros((nv.value, 3))
    T = np.zeros((nf.value, 3), dtype=np.uint32)
    _check(lib.shl_icosphere(level, X.ctypes.data, nv.value, T.ctypes.data, nf.value, ctypes.byref(nv),
                             ctypes.byref(nf)), "shl_icosphere")
    return X, T


def icosphere_off(level):
    lib = load()
    n = ctypes.c_size_t()
    _check(lib.shl_icosphere_off(level, None, 0, ctypes.byref(n)), "shl_icosphere_off")
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib.shl_icosphere_off(level, buf, n.value + 1, ctypes.byref(n)), "shl_icosphere_off")
    return buf.value.decode()


def read_off(path):
    lib = load()
    nv, nf = _u32(), _u32()
    _check(lib.shl_read_off(path.encode(), None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nf)), "shl_read_off")
    X = np.zeros((nv.value, 3))
    T = np.zeros((nf.value, 3), dtype=np.uint32)
    _check(lib.shl_read_off(path.encode(), X.ctypes.data, nv.value, T.ctypes.data, nf.value, ctypes.byref(nv),
                            ctypes.byref(nf)), "shl_read_off")
    return X, T


def gaussian_normal_imperfection(X, amplitude, seed):
    lib = load()
    X = np.ascontiguousarray(X, dtype=np.float64)
    u = np.zeros_like(X)
    _check(lib.shl_gaussian_normal_imperfection(X.ctypes.data, X.shape[0], amplitude, seed, u.ctypes.data),
           "shl_gaussian_normal_imperfection")
    return u


def measure_fp64_peak():
    lib = load()
    t = _d()
    _check(lib.shl_measure_fp64_peak(ctypes.byref(t)), "shl_measure_fp64_peak", False)
    return t.value


def make_mesh(X, T):
    X = np.ascontiguousarray(X, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.uint32)
    m = ShlMesh(X.shape[0], T.shape[0], X.ctypes.data, T.ctypes.data)
    return m, (X, T)


class Shell:
    """One shell on the current CUDA device (mirror of ShellSystem's step API)."""

    def __init__(self, X, T, params):
        lib = load()
        self.lib = lib
        self.params = params
        m, keep = make_mesh(X, T)
        self.X, self.T = keep
        self.V, self.F = self.X.shape[0], self.T.shape[0]
        h = ctypes.c_void_p()
        _check(lib.shl_create(ctypes.byref(m), ctypes.byref(params), ctypes.byref(h)), "shl_create", False)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.shl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- ShellSystem::apply_initial_conditions
    def apply_initial_conditions(self, u0, t0=0.0, pressure_next=None):
        u0 = np.ascontiguousarray(u0, dtype=np.float64).reshape(-1)
        p = self.params.pressure if pressure_next is None else pressure_next
        return _check(self.lib.shl_apply_initial_conditions(self.h, u0.ctypes.data, t0, p),
                      "shl_apply_initial_conditions")

    def set_state(self, u=None, v=None, a=None):
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (u, v, a)]
        return _check(self.lib.shl_set_state(self.h, *[_ptr(x) for x in arrs]), "shl_set_state", False)

    def get_state(self, out=None):
        """Returns (u, v, a); with out=(u, v, a) (contiguous float64 arrays of 3 V values, e.g. views of
        pinned host buffers) the state is copied into them."""
        if out is None:
            u, v, a = (np.zeros(3 * self.V) for _ in range(3))
        else:
            u, v, a = out
            for x in out:
                if x.dtype != np.float64 or x.size != 3 * self.V or not x.flags.c_contiguous:
                    raise ValueError("get_state: out arrays must be contiguous float64 of %d values" % (3 * self.V))
        _check(self.lib.shl_get_state(self.h, u.ctypes.data, v.ctypes.data, a.ctypes.data), "shl_get_state", False)
        return u, v, a

    def set_time(self, t, step):
        _check(self.lib.shl_set_time(self.h, t, step), "shl_set_time", False)

    def get_time(self):
        t, s = _d(), _u32()
        _check(self.lib.shl_get_time(self.h, ctypes.byref(t), ctypes.byref(s)), "shl_get_time", False)
        return t.value, s.value

    def eval_forces(self, u_pred, v_pred, pressure):
        u_pred = np.ascontiguousarray(u_pred, dtype=np.float64).reshape(-1)
        v_pred = np.ascontiguousarray(v_pred, dtype=np.float64).reshape(-1)
        f = np.zeros(3 * self.V)
        a = np.zeros(3 * self.V)
        e = ShlEnergies()
        st = _check(self.lib.shl_eval_forces(self.h, u_pred.ctypes.data, v_pred.ctypes.data, pressure, f.ctypes.data,
                                             a.ctypes.data, ctypes.byref(e)), "shl_eval_forces")
        return f, a, e.as_dict(), st

    # --- n x ShellSystem::advance
    def step(self, n, pressure_table=None, use_graph=True):
        r = ShlStepReport()
        pt = None if pressure_table is None else np.ascontiguousarray(pressure_table, dtype=np.float64)
        st = _check(self.lib.shl_step(self.h, n, _ptr(pt), 1 if use_graph else 0, ctypes.byref(r)), "shl_step")
        return r, st

    # --- asynchronous stepping (CUDA-event timing on the context stream)
    def stream_handle(self):
        h = ctypes.c_void_p()
        _check(self.lib.shl_get_stream(self.h, ctypes.byref(h)), "shl_get_stream", False)
        return h.value or 0

    def upload_pressure_table(self, table):
        t = np.ascontiguousarray(table, dtype=np.float64)
        _check(self.lib.shl_upload_pressure_table(self.h, t.ctypes.data, t.size), "shl_upload_pressure_table", False)

    def step_enqueue(self, n):
        _check(self.lib.shl_step_enqueue(self.h, n), "shl_step_enqueue", False)

    def step_collect(self):
        r = ShlStepReport()
        st = _check(self.lib.shl_step_collect(self.h, ctypes.byref(r)), "shl_step_collect")
        return r, st

    PHASES = ("predict", "cells1", "elements", "contact", "gather_correct", "cells2", "volume_end")

    def profile_step(self, pressure, flush_bytes=0):
        out = np.zeros(7)
        _check(self.lib.shl_profile_step(self.h, pressure, flush_bytes, out.ctypes.data), "shl_profile_step", False)
        return dict(zip(self.PHASES, out))

    def time_kernel(self, which, reps=20, flush_bytes=0):
        ms = _d()
        _check(self.lib.shl_time_kernel(self.h, which, reps, flush_bytes, ctypes.byref(ms)), "shl_time_kernel", False)
        return ms.value

    def contact_state(self):
        n = ctypes.c_size_t()
        du = _d()
        _check(self.lib.shl_get_contact_state(self.h, None, None, None, None, 0, ctypes.byref(n), ctypes.byref(du)),
               "shl_get_contact_state", False)
        k = n.value
        pairs = np.zeros((k, 2), dtype=np.uint32)
        stick = np.zeros(k, dtype=np.uint8)
        orig = np.zeros((k, 3))
        d2 = np.zeros(k)
        if k:
            _check(self.lib.shl_get_contact_state(self.h, pairs.ctypes.data, stick.ctypes.data, orig.ctypes.data,
                                                  d2.ctypes.data, k, ctypes.byref(n), ctypes.byref(du)),
                   "shl_get_contact_state", False)
        return {"pairs": pairs, "stick": stick, "origin": orig, "d2": d2, "du_sum": du.value}

    def set_contact_state(self, pairs, stick=None, origin=None, d2=None, du_sum=0.0):
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        k = pairs.shape[0]
        stick = None if stick is None else np.ascontiguousarray(stick, dtype=np.uint8)
        origin = None if origin is None else np.ascontiguousarray(origin, dtype=np.float64)
        d2 = None if d2 is None else np.ascontiguousarray(d2, dtype=np.float64)
        _check(self.lib.shl_set_contact_state(self.h, pairs.ctypes.data, _ptr(stick), _ptr(origin), _ptr(d2), k,
                                              du_sum), "shl_set_contact_state", False)

    def contact_coords(self):
        """SMOOTH contact: (n_pairs, 4) closest-point coordinates (v1, w1, v2, w2), patch frames."""
        n = ctypes.c_size_t()
        _check(self.lib.shl_get_contact_coords(self.h, None, 0, ctypes.byref(n)), "shl_get_contact_coords", False)
        x = np.zeros((n.value, 4))
        if n.value:
            _check(self.lib.shl_get_contact_coords(self.h, x.ctypes.data, n.value, ctypes.byref(n)),
                   "shl_get_contact_coords", False)
        return x

    def set_contact_coords(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 4)
        _check(self.lib.shl_set_contact_coords(self.h, x.ctypes.data, x.shape[0]), "shl_set_contact_coords", False)

    def rebuild_contacts(self):
        return _check(self.lib.shl_rebuild_contacts(self.h), "shl_rebuild_contacts")

    def element_fields(self):
        out = [np.zeros(self.F) for _ in range(5)]
        _check(self.lib.shl_get_element_fields(self.h, *[o.ctypes.data for o in out]), "shl_get_element_fields",
               False)
        return dict(zip(("kGauss", "kMean", "etens", "ebend", "area"), out))

    def mass_damping(self):
        Minv, C = np.zeros(3 * self.V), np.zeros(3 * self.V)
        _check(self.lib.shl_get_mass_damping(self.h, Minv.ctypes.data, C.ctypes.data), "shl_get_mass_damping", False)
        return Minv, C

    n_shells = 1  # a Batch sets its own count

    def set_pressure_function(self, expr):
        """Pressure as an expression of t evaluated on the device each step (None: use the table)."""
        _check(self.lib.shl_set_pressure_function(self.h, None if expr is None else expr.encode()),
               "shl_set_pressure_function", False)

    def set_stop_function(self, expr):
        """Stopping criterion (expression of t) tested on the device after every step (None: none)."""
        _check(self.lib.shl_set_stop_function(self.h, None if expr is None else expr.encode()),
               "shl_set_stop_function", False)

    def set_cavity_functions(self, rx=None, ry=None, rz=None):
        """Cavity semi-axes as expressions of t (None keeps the constant)."""
        enc = lambda e: None if e is None else e.encode()  # noqa: E731
        _check(self.lib.shl_set_cavity_functions(self.h, enc(rx), enc(ry), enc(rz)), "shl_set_cavity_functions",
               False)

    def set_element_variant(self, v):
        _check(self.lib.shl_set_element_variant(self.h, v), "shl_set_element_variant", False)

    def element_variant(self):
        """(variant id, name, tuning times in ms of all variants)."""
        v = ctypes.c_int()
        name = ctypes.create_string_buffer(64)
        ms = np.zeros(ELEMENT_VARIANTS, dtype=np.float32)
        _check(self.lib.shl_get_element_variant(self.h, ctypes.byref(v), name, 64, ms.ctypes.data),
               "shl_get_element_variant", False)
        return v.value, name.value.decode(), ms

    def scale_damping(self, factor):
        _check(self.lib.shl_scale_damping(self.h, factor), "shl_scale_damping", False)

    def cavity_origins(self):
        o = np.zeros(3 * self.V)
        _check(self.lib.shl_get_cavity_origins(self.h, o.ctypes.data), "shl_get_cavity_origins", False)
        return o

    def dt(self):
        """(current dt, repeated attempts since the last report)."""
        d, r = _d(), _u32()
        _check(self.lib.shl_get_dt(self.h, ctypes.byref(d), ctypes.byref(r)), "shl_get_dt", False)
        return d.value, r.value

    def eval_pressure_function(self, t):
        t = np.ascontiguousarray(t, dtype=np.float64)
        out = np.zeros_like(t)
        _check(self.lib.shl_eval_pressure_function(self.h, t.ctypes.data, t.size, out.ctypes.data),
               "shl_eval_pressure_function", False)
        return out

    def residual(self, pressure, flags=0):
        """Relative residual ||f_ext - f_int|| / ||f_ext|| of the stored state, per shell
        (flags: RESIDUAL_FP64, RESIDUAL_CORRECT, RESIDUAL_CLEAR, RESIDUAL_CONTACT)."""
        n = self.n_shells
        rel, f2, e2 = np.zeros(n), np.zeros(n), np.zeros(n)
        _check(self.lib.shl_residual(self.h, pressure, flags, rel.ctypes.data, f2.ctypes.data, e2.ctypes.data),
               "shl_residual", False)
        return rel

    def node_fields(self):
        """Per-node ekin, ecav, eself, efric densities and masses of the last step."""
        out = [np.zeros(self.V) for _ in range(5)]
        _check(self.lib.shl_get_node_fields(self.h, *[o.ctypes.data for o in out]), "shl_get_node_fields", False)
        return dict(zip(("ekin", "ecav", "eself", "efric", "mass"), out))

    def save_state_file(self, path, time_step, dt, wall_time=0.0, avg_rows=None):
        """Write a state file in the layout of ShellSystem::save (see shl_save_state_file)."""
        rows = np.zeros((0, 14)) if avg_rows is None else np.ascontiguousarray(avg_rows, dtype=np.float64)
        _check(self.lib.shl_save_state_file(self.h, os.fsencode(path), time_step, dt, wall_time,
                                            rows.ctypes.data if rows.size else None, rows.shape[0]),
               "shl_save_state_file", False)

    def load_state_file(self, path, max_rows=1 << 16):
        """Load a state file; returns (time_step, dt, wall_time, avg_rows)."""
        step, dt, wt, n = _u32(), _d(), _d(), _u32()
        rows = np.zeros((max_rows, 14))
        _check(self.lib.shl_load_state_file(self.h, os.fsencode(path), ctypes.byref(step), ctypes.byref(dt),
                                            ctypes.byref(wt), rows.ctypes.data, max_rows, ctypes.byref(n)),
               "shl_load_state_file", False)
        return step.value, dt.value, wt.value, rows[:n.value].copy()

    def write_vtu(self, path):
        """ASCII .vtu of the current state (ShellSystem::write_vtk)."""
        _check(self.lib.shl_write_vtu(self.h, os.fsencode(path)), "shl_write_vtu", False)


class Batch(Shell):
    """Independent shells advanced together (shl_batch_create)."""

    def __init__(self, meshes, params, pressure_scale=None):
        lib = load()
        self.lib = lib
        self.params = params[0]
        n = len(meshes)
        keep = [make_mesh(X, T) for X, T in meshes]
        arr = (ShlMesh * n)(*[m for m, _ in keep])
        parr = (ShlParams * n)(*params)
        ps = None if pressure_scale is None else np.ascontiguousarray(pressure_scale, dtype=np.float64)
        h = ctypes.c_void_p()
        _check(lib.shl_batch_create(ctypes.cast(arr, ctypes.c_void_p), ctypes.cast(parr, ctypes.c_void_p),
                                    _ptr(ps), n, ctypes.byref(h)), "shl_batch_create", False)
        self.h = h
        self.n_shells = n
        no = np.zeros(n + 1, dtype=np.uint32)
        fo = np.zeros(n + 1, dtype=np.uint32)
        _check(lib.shl_batch_layout(h, None, no.ctypes.data, fo.ctypes.data), "shl_batch_layout", False)
        self.node_off, self.face_off = no.astype(np.int64), fo.astype(np.int64)
        self.V, self.F = int(no[-1]), int(fo[-1])
        self.X = np.concatenate([np.asarray(X, float).reshape(-1, 3) for X, _ in meshes])
        self.T = np.concatenate([np.asarray(T, np.int64) + no[k] for k, (_, T) in enumerate(meshes)])

    def split(self, vec):
        """Per-shell views of a concatenated node-major vector."""
        return [vec[3 * self.node_off[k]:3 * self.node_off[k + 1]] for k in range(self.n_shells)]

    def contact_stats(self):
        """Per shell (self-contact on): du_sum and the candidate-list rebuilds since creation."""
        du = np.zeros(self.n_shells)
        nr = np.zeros(self.n_shells, dtype=np.uint32)
        _check(self.lib.shl_batch_contact_stats(self.h, du.ctypes.data, nr.ctypes.data), "shl_batch_contact_stats",
               False)
        return du, nr

    def split_pairs(self, pairs):
        """Contact pairs (batch face ids) per shell, in each shell's own face ids."""
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        shell = np.searchsorted(self.face_off, pairs[:, 0], side="right") - 1
        return [pairs[shell == k] - self.face_off[k] for k in range(self.n_shells)]


def gemm_bf16(A_bits, B_bits):
    """C = A . B^T through the library's BF16 GEMM (A, B: uint16 BF16 bit patterns)."""
    lib = load()
    A_bits = np.ascontiguousarray(A_bits, dtype=np.uint16)
    B_bits = np.ascontiguousarray(B_bits, dtype=np.uint16)
    M, K = A_bits.shape
    N = B_bits.shape[0]
    C = np.zeros((M, N), dtype=np.float32)
    _check(lib.shl_gemm_bf16(A_bits.ctypes.data, B_bits.ctypes.data, M, N, K, C.ctypes.data), "shl_gemm_bf16", False)
    return C


def gemm_bf16_time(M, N, K, reps=20):
    """Average device ms of the library's BF16 GEMM (M x K) . (N x K)^T on device-resident operands."""
    lib = load()
    ms = _d()
    _check(lib.shl_gemm_bf16_time(M, N, K, reps, ctypes.byref(ms)), "shl_gemm_bf16_time", False)
    return ms.value


class MLP:
    """The warm-start surrogate network (shl_mlp_*): dims[0] -> ... -> dims[-1], GELU between layers."""

    def __init__(self, dims, max_batch=256, seed=0):
        self.lib = load()
        self.dims = [int(d) for d in dims]
        arr = (_u32 * len(self.dims))(*self.dims)
        h = ctypes.c_void_p()
        _check(self.lib.shl_mlp_create(arr, len(self.dims), max_batch, seed, ctypes.byref(h)), "shl_mlp_create", False)
        self.h = h
        self.max_batch = max_batch

    def close(self):
        if getattr(self, "h", None):
            self.lib.shl_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        out = []
        for l in range(len(self.dims) - 1):
            W = np.zeros((self.dims[l + 1], self.dims[l]), dtype=np.float32)
            b = np.zeros(self.dims[l + 1], dtype=np.float32)
            _check(self.lib.shl_mlp_get_params(self.h, l, W.ctypes.data, b.ctypes.data), "shl_mlp_get_params", False)
            out.append((W, b))
        return out

    def set_params(self, params):
        for l, (W, b) in enumerate(params):
            W = np.ascontiguousarray(W, dtype=np.float32)
            b = np.ascontiguousarray(b, dtype=np.float32)
            _check(self.lib.shl_mlp_set_params(self.h, l, W.ctypes.data, b.ctypes.data), "shl_mlp_set_params", False)

    def set_dataset(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        self._data = (X, T)
        _check(self.lib.shl_mlp_set_dataset(self.h, X.ctypes.data, T.ctypes.data, X.shape[0]), "shl_mlp_set_dataset",
               False)

    def train(self, iters, batch, lr0=1e-3, lr_final=1e-5, seed=0, curve_every=100):
        curve = np.zeros((iters + curve_every - 1) // curve_every, dtype=np.float32)
        _check(self.lib.shl_mlp_train(self.h, iters, batch, lr0, lr_final, seed, curve.ctypes.data, curve_every),
               "shl_mlp_train", False)
        return curve

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.dims[-1]), dtype=np.float32)
        _check(self.lib.shl_mlp_predict(self.h, X.ctypes.data, X.shape[0], Y.ctypes.data), "shl_mlp_predict", False)
        return Y

    def gradients(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        L = len(self.dims) - 1
        dW = [np.zeros((self.dims[l + 1], self.dims[l]), dtype=np.float32) for l in range(L)]
        db = [np.zeros(self.dims[l + 1], dtype=np.float32) for l in range(L)]
        pW = (ctypes.c_void_p * L)(*[w.ctypes.data for w in dW])
        pb = (ctypes.c_void_p * L)(*[b.ctypes.data for b in db])
        loss = _d()
        _check(self.lib.shl_mlp_gradients(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], ctypes.byref(loss), pW, pb),
               "shl_mlp_gradients", False)
        return loss.value, dW, db
