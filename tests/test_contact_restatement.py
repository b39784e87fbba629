"""The library's narrow phase and friction law against the oracle's restatement.

The library's shl_pair_compute / shl_friction_apply (shell_gb300/csrc/shl_geom.h,
used by the CUDA kernels with separately rounded operations) and the oracle's
restatement of ShellShellContact::compute (ShellShellContact.C:35-145) and
Friction::apply (Friction.C:4-60), written on its own vector type, must agree
bit for bit: the candidate lists and friction states of the GPU parity tests
depend on it.  The library's host build of the header is compiled here into a
small harness (g++, -ffp-contract=off, as the library's host code is built).
Inputs: random triangle pairs at all scales of separation, and degenerate
configurations (shared vertices, parallel and collinear edges, coplanar faces,
touching triangles); friction states in all four transitions.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = r'''
#include "shl_geom.h"
extern "C" void lib_pair_compute(const double* p, double* out) {
  const double* p1[3] = {p, p + 3, p + 6};
  const double* p2[3] = {p + 9, p + 12, p + 15};
  shl_pair_geom g;
  shl_pair_compute(p1, p2, &g);
  out[0] = g.d2; out[1] = g.dc[0]; out[2] = g.dc[1]; out[3] = g.dc[2];
  out[4] = g.v[0]; out[5] = g.w[0]; out[6] = g.v[1]; out[7] = g.w[1];
}
extern "C" void lib_friction_apply(double* E, double* fc, double fn, const double* n, const double* v, double avn,
                                   double vs, double k, double mus, double mud, double damp, int* stick,
                                   double* so, const double* cp) {
  shl_friction_apply(E, fc, fn, n, v, avn, vs, k, mus, mud, damp, stick, so, cp);
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("geom")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    so = d / "libh.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "shell_gb300", "csrc"), str(src), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    vp, d_ = ctypes.c_void_p, ctypes.c_double
    lib.lib_pair_compute.argtypes = [vp, vp]
    lib.lib_friction_apply.argtypes = [vp, vp, d_, vp, vp, d_, d_, d_, d_, d_, d_, vp, vp, vp]
    return lib


def _pairs(rng, n):
    out = []
    for k in range(n):
        scale = 10.0 ** rng.uniform(-6, 0)
        t1 = rng.standard_normal((3, 3))
        t2 = t1.mean(axis=0) + scale * rng.standard_normal(3) + rng.standard_normal((3, 3)) * rng.uniform(0.1, 1)
        kind = k % 8
        if kind == 1:      # shared vertex
            t2[0] = t1[1]
        elif kind == 2:    # shared edge
            t2[0], t2[1] = t1[1], t1[0]
        elif kind == 3:    # parallel edges
            t2[1] = t2[0] + (t1[1] - t1[0]) * 0.7
        elif kind == 4:    # coplanar
            nrm = np.cross(t1[1] - t1[0], t1[2] - t1[0])
            nrm /= np.linalg.norm(nrm)
            t2 -= np.outer((t2 - t1[0]) @ nrm, nrm)
        elif kind == 5:    # collinear edge with a vertex of the other
            t2[2] = t1[0] + 0.5 * (t1[1] - t1[0])
        elif kind == 6:    # degenerate (zero-area) triangle
            t2[2] = t2[1]
        out.append(np.concatenate([t1.ravel(), t2.ravel()]))
    return out


def test_pair_compute_bitexact(harness):
    O.load()
    rng = np.random.default_rng(5)
    ours, theirs = np.zeros(8), np.zeros(8)
    for p in _pairs(rng, 20000):
        p = np.ascontiguousarray(p)
        harness.lib_pair_compute(p.ctypes.data, ours.ctypes.data)
        r = O.pair_compute(p[:9].reshape(3, 3), p[9:].reshape(3, 3))
        theirs[:] = [r["d2"], *r["dc"], r["v"][0], r["w"][0], r["v"][1], r["w"][1]]
        # d2 and dc bit for bit; barycentrics by value (+0 and -0 are the same point)
        assert np.array_equal(ours[:4].view(np.uint64), theirs[:4].view(np.uint64)), p
        assert np.array_equal(ours[4:], theirs[4:]), p


def test_friction_bitexact(harness):
    rng = np.random.default_rng(9)
    counts = {}
    for k in range(20000):
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        v = rng.standard_normal(3) * 10.0 ** rng.uniform(-4, 0)
        avn = float(v @ n)
        v_stop = 0.03
        kk = 10.0 ** rng.uniform(-2, 3)
        mu_s, mu_d = (0.3, 0.3) if k % 3 else (0.0, 0.2)
        damping = 0.0 if k % 2 else 0.01
        fn = 10.0 ** rng.uniform(-6, -1)
        stick0 = int(rng.random() < 0.5)
        so0 = rng.standard_normal(3) * 1e-3 * stick0
        cp = rng.standard_normal(3) * 1e-3
        res = []
        for fun in ("lib", "oracle"):
            E = ctypes.c_double(0.0)
            fc = np.zeros(3)
            st = ctypes.c_int(stick0)
            so = so0.copy()
            args = [fc.ctypes.data, fn, n.ctypes.data, v.ctypes.data, avn, v_stop, kk, mu_s, mu_d, damping]
            if fun == "lib":
                harness.lib_friction_apply(ctypes.byref(E), *args, ctypes.byref(st), so.ctypes.data, cp.ctypes.data)
                res.append((E.value, fc.copy(), st.value, so.copy()))
            else:
                res.append(O.friction_apply(fn, n, v, avn, v_stop, kk, mu_s, mu_d, damping, stick0, so0, cp))
        (E1, f1, s1, o1), (E2, f2, s2, o2) = res[0], (res[1][0], res[1][1], res[1][2], res[1][3])
        assert s1 == s2 and E1 == E2
        assert np.array_equal(f1.view(np.uint64), f2.view(np.uint64))
        assert np.array_equal(o1, o2)
        counts[(stick0, s1)] = counts.get((stick0, s1), 0) + 1
    # every transition of the slip-stick state machine was exercised
    assert all(counts.get(t, 0) > 100 for t in ((0, 0), (0, 1), (1, 0), (1, 1))), counts
