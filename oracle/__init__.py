"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA library.
Only the tests, `__graft_entry__.smoke()` and the CPU-baseline leg of
`bench.py` load it; the library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    args = ["make", "-C", HERE]
    if force:
        subprocess.run(["make", "-C", HERE, "clean"], check=True, stdout=subprocess.DEVNULL)
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode(errors="replace"))
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    from shell_gb300.abi import ShlEnergies, ShlMesh, ShlParams, ShlStepReport

    lib = ctypes.CDLL(LIB_PATH)
    vp, d, u32, sz = ctypes.c_void_p, ctypes.c_double, ctypes.c_uint32, ctypes.c_size_t
    sig = {
        "oracle_error": (ctypes.c_char_p, []),
        "oracle_set_threads": (None, [ctypes.c_int]),
        "oracle_create": (vp, [ctypes.POINTER(ShlMesh), ctypes.POINTER(ShlParams)]),
        "oracle_destroy": (None, [vp]),
        "oracle_apply_initial_conditions": (ctypes.c_int, [vp, vp, d, d]),
        "oracle_set_state": (ctypes.c_int, [vp, vp, vp, vp]),
        "oracle_get_state": (ctypes.c_int, [vp, vp, vp, vp]),
        "oracle_set_time": (ctypes.c_int, [vp, d, u32]),
        "oracle_get_time": (ctypes.c_int, [vp, ctypes.POINTER(d), ctypes.POINTER(u32)]),
        "oracle_eval_forces": (ctypes.c_int, [vp, vp, vp, d, vp, vp, ctypes.POINTER(ShlEnergies)]),
        "oracle_step": (ctypes.c_int, [vp, u32, vp, ctypes.POINTER(ShlStepReport)]),
        "oracle_get_contact_state": (sz, [vp, vp, vp, vp, vp, sz, ctypes.POINTER(d)]),
        "oracle_set_contact_state": (ctypes.c_int, [vp, vp, vp, vp, vp, sz, d]),
        "oracle_rebuild_contacts": (ctypes.c_int, [vp]),
        "oracle_get_mass_damping": (ctypes.c_int, [vp, vp, vp]),
        "oracle_get_element_fields": (ctypes.c_int, [vp, vp, vp, vp, vp, vp]),
        "oracle_get_cell_info": (ctypes.c_int, [vp, vp]),
        "oracle_get_node_fields": (ctypes.c_int, [vp, vp, vp, vp]),
        "oracle_set_pressure_function": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "oracle_get_dt": (d, [vp]),
        "oracle_set_cavity_functions": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]),
        "oracle_get_cavity": (ctypes.c_int, [vp, vp, vp, vp]),
        "oracle_get_rejections": (ctypes.c_uint64, [vp]),
        "oracle_patch": (ctypes.c_int, [vp, u32, vp, ctypes.POINTER(u32)]),
        "oracle_get_contact_coords": (sz, [vp, vp, sz]),
        "oracle_set_contact_coords": (ctypes.c_int, [vp, vp, sz]),
        "oracle_limit_eval": (ctypes.c_int, [vp, u32, d, d, vp]),
        "oracle_limit_basis": (ctypes.c_int, [vp, u32, d, d, vp]),
        "oracle_smooth_closest": (ctypes.c_int, [vp, u32, u32, vp, ctypes.POINTER(d), vp]),
        "oracle_subdiv_table": (sz, [ctypes.c_int, vp, sz]),
        "oracle_basis_at": (ctypes.c_int, [vp, u32, d, d, vp]),
        "oracle_basis_cached": (ctypes.c_int, [vp, u32, vp, vp]),
        "oracle_elem_metric": (ctypes.c_int, [vp, u32, ctypes.c_int, vp]),
        "oracle_close_elems": (ctypes.c_int, [vp, u32, vp, sz, ctypes.POINTER(sz)]),
        "oracle_segment_segment": (None, [vp, vp, vp, vp, vp, vp]),
        "oracle_point_triangle": (None, [vp, vp, vp, vp, vp, vp]),
        "oracle_pair_compute": (None, [vp, vp]),
        "oracle_friction_apply": (None, [vp, vp, d, vp, vp, d, d, d, d, d, d, ctypes.POINTER(ctypes.c_int), vp, vp]),
        "oracle_fixed_order_sum": (d, [vp, u32]),
        "oracle_fp_contract_off": (ctypes.c_int, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class Oracle:
    """CPU restatement of one ShellSystem (FP64)."""

    def __init__(self, X, T, params, threads=None):
        from shell_gb300.abi import ShlMesh

        self.lib = load()
        if threads is not None:
            self.lib.oracle_set_threads(threads)
        X = np.ascontiguousarray(X, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.uint32)
        m = ShlMesh(X.shape[0], T.shape[0], X.ctypes.data, T.ctypes.data)
        self.X, self.T = X, T
        self.V, self.F = self.X.shape[0], self.T.shape[0]
        self.params = params
        self.h = self.lib.oracle_create(ctypes.byref(m), ctypes.byref(params))
        if not self.h:
            raise RuntimeError("oracle_create: " + self.lib.oracle_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply_initial_conditions(self, u0, t0=0.0, pressure_next=None):
        u0 = np.ascontiguousarray(u0, dtype=np.float64).reshape(-1)
        p = self.params.pressure if pressure_next is None else pressure_next
        return self.lib.oracle_apply_initial_conditions(self.h, u0.ctypes.data, t0, p)

    def set_state(self, u=None, v=None, a=None):
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (u, v, a)]
        return self.lib.oracle_set_state(self.h, *[None if x is None else x.ctypes.data for x in arrs])

    def get_state(self):
        u, v, a = (np.zeros(3 * self.V) for _ in range(3))
        self.lib.oracle_get_state(self.h, u.ctypes.data, v.ctypes.data, a.ctypes.data)
        return u, v, a

    def set_time(self, t, step):
        self.lib.oracle_set_time(self.h, t, step)

    def get_time(self):
        t, s = ctypes.c_double(), ctypes.c_uint32()
        self.lib.oracle_get_time(self.h, ctypes.byref(t), ctypes.byref(s))
        return t.value, s.value

    def eval_forces(self, u_pred, v_pred, pressure):
        from shell_gb300.abi import ShlEnergies

        u_pred = np.ascontiguousarray(u_pred, dtype=np.float64).reshape(-1)
        v_pred = np.ascontiguousarray(v_pred, dtype=np.float64).reshape(-1)
        f, a = np.zeros(3 * self.V), np.zeros(3 * self.V)
        e = ShlEnergies()
        st = self.lib.oracle_eval_forces(self.h, u_pred.ctypes.data, v_pred.ctypes.data, pressure, f.ctypes.data,
                                         a.ctypes.data, ctypes.byref(e))
        return f, a, e.as_dict(), st

    def step(self, n, pressure_table=None):
        from shell_gb300.abi import ShlStepReport

        r = ShlStepReport()
        pt = None if pressure_table is None else np.ascontiguousarray(pressure_table, dtype=np.float64)
        st = self.lib.oracle_step(self.h, n, None if pt is None else pt.ctypes.data, ctypes.byref(r))
        return r, st

    def contact_state(self):
        du = ctypes.c_double()
        k = self.lib.oracle_get_contact_state(self.h, None, None, None, None, 0, ctypes.byref(du))
        pairs = np.zeros((k, 2), dtype=np.uint32)
        stick = np.zeros(k, dtype=np.uint8)
        orig = np.zeros((k, 3))
        d2 = np.zeros(k)
        if k:
            self.lib.oracle_get_contact_state(self.h, pairs.ctypes.data, stick.ctypes.data, orig.ctypes.data,
                                              d2.ctypes.data, k, ctypes.byref(du))
        return {"pairs": pairs, "stick": stick, "origin": orig, "d2": d2, "du_sum": du.value}

    def set_contact_state(self, pairs, stick=None, origin=None, d2=None, du_sum=0.0):
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        k = pairs.shape[0]
        ptr = lambda a, dt: None if a is None else np.ascontiguousarray(a, dtype=dt).ctypes.data  # noqa: E731
        keep = [np.ascontiguousarray(x, dtype=t) if x is not None else None
                for x, t in ((stick, np.uint8), (origin, np.float64), (d2, np.float64))]
        r = self.lib.oracle_set_contact_state(self.h, pairs.ctypes.data, *[None if x is None else x.ctypes.data
                                                                           for x in keep], k, du_sum)
        del ptr
        if r != 0:
            raise RuntimeError(self.lib.oracle_error().decode())

    def rebuild_contacts(self):
        return self.lib.oracle_rebuild_contacts(self.h)

    def mass_damping(self):
        Minv, C = np.zeros(3 * self.V), np.zeros(3 * self.V)
        self.lib.oracle_get_mass_damping(self.h, Minv.ctypes.data, C.ctypes.data)
        return Minv, C

    def element_fields(self):
        out = [np.zeros(self.F) for _ in range(5)]
        self.lib.oracle_get_element_fields(self.h, *[o.ctypes.data for o in out])
        return dict(zip(("kGauss", "kMean", "etens", "ebend", "area"), out))

    def set_pressure_function(self, expr):
        if self.lib.oracle_set_pressure_function(self.h, None if expr is None else expr.encode()) != 0:
            raise RuntimeError(self.lib.oracle_error().decode())

    def dt(self):
        return self.lib.oracle_get_dt(self.h)

    def set_cavity_functions(self, rx=None, ry=None, rz=None):
        enc = lambda e: None if e is None else e.encode()  # noqa: E731
        if self.lib.oracle_set_cavity_functions(self.h, enc(rx), enc(ry), enc(rz)) != 0:
            raise RuntimeError(self.lib.oracle_error().decode())

    def cavity(self):
        o, e, t = np.zeros(3 * self.V), np.zeros(self.V), np.zeros(3)
        self.lib.oracle_get_cavity(self.h, o.ctypes.data, e.ctypes.data, t.ctypes.data)
        return {"origins": o, "ecav": e, "Ecav": t[0], "cavity_force": t[1], "Nc_cav": int(t[2])}

    def rejections(self):
        return int(self.lib.oracle_get_rejections(self.h))

    def node_fields(self):
        out = [np.zeros(self.V) for _ in range(3)]
        self.lib.oracle_get_node_fields(self.h, *[o.ctypes.data for o in out])
        return dict(zip(("ekin", "eself", "efric"), out))

    def cell_info(self):
        out = np.zeros(9)
        self.lib.oracle_get_cell_info(self.h, out.ctypes.data)
        return {"avg_elem_size": out[0], "cell_size": out[1], "d_max": out[2], "bmin": out[3:6], "bmax": out[6:9]}

    def patch(self, eid):
        nodes = np.zeros(18, dtype=np.uint32)
        n = ctypes.c_uint32()
        self.lib.oracle_patch(self.h, eid, nodes.ctypes.data, ctypes.byref(n))
        return nodes[:n.value].copy()

    def contact_coords(self):
        k = self.lib.oracle_get_contact_coords(self.h, None, 0)
        x = np.zeros((k, 4))
        if k:
            self.lib.oracle_get_contact_coords(self.h, x.ctypes.data, k)
        return x

    def set_contact_coords(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 4)
        if self.lib.oracle_set_contact_coords(self.h, x.ctypes.data, x.shape[0]) != 0:
            raise RuntimeError(self.lib.oracle_error().decode())

    def limit_eval(self, eid, v, w):
        """SMOOTH: point and first / second derivatives of the limit surface, (6, 3)."""
        out = np.zeros(18)
        if self.lib.oracle_limit_eval(self.h, eid, v, w, out.ctypes.data) != 0:
            raise RuntimeError(self.lib.oracle_error().decode())
        return out.reshape(6, 3)

    def limit_basis(self, eid, v, w):
        """SMOOTH: limit-surface weights of the patch nodes at (v, w), (N + 6, 6)."""
        n = len(self.patch(eid))
        out = np.zeros(6 * n)
        if self.lib.oracle_limit_basis(self.h, eid, v, w, out.ctypes.data) != 0:
            raise RuntimeError(self.lib.oracle_error().decode())
        return out.reshape(n, 6)

    def smooth_closest(self, e1, e2, x0=(1 / 3, 1 / 3, 1 / 3, 1 / 3)):
        x = np.array(x0, dtype=np.float64)
        d2 = ctypes.c_double()
        dc = np.zeros(3)
        it = self.lib.oracle_smooth_closest(self.h, e1, e2, x.ctypes.data, ctypes.byref(d2), dc.ctypes.data)
        if it < 0:
            raise RuntimeError(self.lib.oracle_error().decode())
        return x, d2.value, dc, it

    def basis_at(self, eid, v, w):
        n = len(self.patch(eid))
        out = np.zeros(6 * n)
        self.lib.oracle_basis_at(self.h, eid, v, w, out.ctypes.data)
        return out.reshape(n, 6)

    def basis_cached(self, eid):
        n = len(self.patch(eid))
        out = np.zeros(6 * n)
        R = np.zeros(4)
        self.lib.oracle_basis_cached(self.h, eid, out.ctypes.data, R.ctypes.data)
        return out.reshape(n, 6), R.reshape(2, 2)

    def elem_metric(self, eid, which=0):
        out = np.zeros(29)
        self.lib.oracle_elem_metric(self.h, eid, which, out.ctypes.data)
        return {"xyz": out[0:3], "vec": out[3:12].reshape(3, 3), "dvec": out[12:21].reshape(3, 3),
                "ff1": out[21:24], "ff2": out[24:27], "jac": out[27], "JxW": out[28]}

    def close_elems(self, eid):
        out = np.zeros(4096, dtype=np.uint32)
        n = ctypes.c_size_t()
        self.lib.oracle_close_elems(self.h, eid, out.ctypes.data, out.size, ctypes.byref(n))
        return out[:n.value].copy()


def segment_segment(p10, p11, p20, p21):
    lib = load()
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (p10, p11, p20, p21)]
    dv, st = np.zeros(3), np.zeros(2)
    lib.oracle_segment_segment(*[x.ctypes.data for x in a], dv.ctypes.data, st.ctypes.data)
    return dv, st


def point_triangle(p0, p1, p2, p3):
    lib = load()
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (p0, p1, p2, p3)]
    dv, vw = np.zeros(3), np.zeros(2)
    lib.oracle_point_triangle(*[x.ctypes.data for x in a], dv.ctypes.data, vw.ctypes.data)
    return dv, vw


def pair_compute(tri1, tri2):
    lib = load()
    p = np.ascontiguousarray(np.concatenate([np.asarray(tri1, float).ravel(), np.asarray(tri2, float).ravel()]))
    out = np.zeros(8)
    lib.oracle_pair_compute(p.ctypes.data, out.ctypes.data)
    return {"d2": out[0], "dc": out[1:4], "v": out[[4, 6]], "w": out[[5, 7]]}


def friction_apply(f_normal, n, v, abs_v_normal, v_stop, k, mu_s, mu_d, damping, stick, spring_origin,
                   contact_point):
    lib = load()
    E = ctypes.c_double()
    fc = np.zeros(3)
    st = ctypes.c_int(int(stick))
    so = np.ascontiguousarray(spring_origin, dtype=np.float64).copy()
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (n, v, contact_point)]
    lib.oracle_friction_apply(ctypes.byref(E), fc.ctypes.data, f_normal, arr[0].ctypes.data, arr[1].ctypes.data,
                              abs_v_normal, v_stop, k, mu_s, mu_d, damping, ctypes.byref(st), so.ctypes.data,
                              arr[2].ctypes.data)
    return E.value, fc, st.value, so


def subdiv_table(N):
    """Subdivision table of valence N: (34, 3, 12, N + 6)."""
    lib = load()
    n = lib.oracle_subdiv_table(N, None, 0)
    out = np.zeros(n)
    lib.oracle_subdiv_table(N, out.ctypes.data, n)
    return out.reshape(34, 3, 12, N + 6)


def fixed_order_sum(x):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib.oracle_fixed_order_sum(x.ctypes.data, x.size)


def fp_contract_off():
    return bool(load().oracle_fp_contract_off())
