"""The library's SMOOTH closest-point search against the oracle's restatement.

The library's search (shell_gb300/csrc/shl_smooth.h: the resumable search
state that k_smooth_search runs, driven here to the end by
shl_smooth_closest) and the oracle's own sequential restatement of the same
active-set projected-Newton method (smooth::closest in
oracle/shell_oracle.cpp), both over the shared limit evaluation
(shl_limit.h), must agree bit for bit: minimiser, squared distance, contact
vector and iteration count.  The library's host build of the headers is
compiled here into a small harness (g++, -ffp-contract=off, as the library's
host code is built).  Inputs: pairs of faces of a squashed icosphere and of
a squashed sphere with valence-5 and valence-7 patches (regular and
irregular patches, faces near and far apart) from the face centres, from
random interior starts and from starts on the edges and vertices of the
triangles.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import cell_size_mult_for, flipped_sphere, physics_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = r'''
#include "shl_limit.h"
#include "shl_smooth.h"
extern "C" int lib_limit_eval(const double* pos, const uint32_t* ids, int N, const double* tab, double v, double w,
                              double* out) {
  shl_limit_patch P = {pos, ids, 1u, N, N == 6 ? 0 : tab};
  double e[6][3];
  shl_limit_eval(&P, v, w, 2, e);
  for (int q = 0; q < 6; ++q)
    for (int c = 0; c < 3; ++c) out[3 * q + c] = e[q][c];
  return 0;
}
extern "C" int lib_smooth_closest(const double* pos, const uint32_t* ida, int na, const double* ta,
                                  const uint32_t* idb, int nb, const double* tb, double* x, double* d2, double* dc) {
  shl_limit_patch A = {pos, ida, 1u, na, na == 6 ? 0 : ta};
  shl_limit_patch B = {pos, idb, 1u, nb, nb == 6 ? 0 : tb};
  return shl_smooth_closest(&A, &B, x, d2, dc);
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("smooth")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    so = d / "libh.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "shell_gb300", "csrc"), str(src), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    vp, d_, i_ = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
    lib.lib_limit_eval.argtypes = [vp, vp, i_, vp, d_, d_, vp]
    lib.lib_smooth_closest.argtypes = [vp, vp, i_, vp, vp, i_, vp, vp, vp, vp]
    lib.lib_smooth_closest.restype = i_
    return lib


@pytest.fixture(scope="module", params=["ico3", "flip"])
def state(request, built):
    X, T = L.icosphere(3) if request.param == "ico3" else flipped_sphere(1)
    p = physics_params(shell_shell_contact=L.CONTACT_SMOOTH, cell_size_mult=cell_size_mult_for(X, T, 0.01))
    o = O.Oracle(X, T, p, threads=2)
    rng = np.random.default_rng(17)
    u = np.zeros_like(X)
    u[:, 2] = (0.0042 - 1.0) * X[:, 2]
    u = (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)
    o.set_state(u, np.zeros_like(u), np.zeros_like(u))
    pos = np.ascontiguousarray((X.reshape(-1) + u), dtype=np.float64)
    tabs = {}
    patches = []
    for e in range(len(T)):
        ids = np.ascontiguousarray(o.patch(e), dtype=np.uint32)
        n = len(ids) - 6
        if n != 6 and n not in tabs:
            tabs[n] = np.ascontiguousarray(O.subdiv_table(n).reshape(-1))
        patches.append((ids, n))
    yield X, T, o, pos, patches, tabs
    o.close()


def _lib_patch(patches, tabs, e):
    ids, n = patches[e]
    tab = tabs.get(n)
    return ids.ctypes.data, n, (tab.ctypes.data if tab is not None else None)


def test_limit_evaluation_positions_agree(harness, state):
    """The harness's positions are the oracle's: its limit evaluation equals
    the oracle's at random points of every face (the shared shl_limit.h)."""
    X, T, o, pos, patches, tabs = state
    rng = np.random.default_rng(3)
    out = np.zeros(18)
    for e in range(0, len(T), 7):
        a = rng.dirichlet([1, 1, 1])
        ids, n, tab = _lib_patch(patches, tabs, e)
        harness.lib_limit_eval(pos.ctypes.data, ids, n, tab, a[1], a[2], out.ctypes.data)
        ref = o.limit_eval(e, a[1], a[2]).reshape(-1)
        assert np.array_equal(out.view(np.uint64), ref.view(np.uint64)), e


def test_search_equals_oracle_restatement(harness, state):
    X, T, o, pos, patches, tabs = state
    rng = np.random.default_rng(11)
    o.rebuild_contacts()
    pairs = [tuple(int(v) for v in q) for q in o.contact_state()["pairs"]]
    assert len(pairs) > 50
    val = np.bincount(T.ravel().astype(int))
    irregular = {e for e in range(len(T)) if (val[T[e].astype(int)] != 6).any()}
    sel = [q for q in pairs if q[0] in irregular or q[1] in irregular][:40] + pairs[::37]
    # far pairs: faces on opposite sides of the sphere
    sel += [(int(e1), int(e2)) for e1, e2 in rng.integers(0, len(T), size=(20, 2)) if e1 != e2]
    corners = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (0.5, 0.0), (0.0, 0.5), (0.5, 0.5)]
    n_irr = n_checked = 0
    for k, (e1, e2) in enumerate(sel):
        starts = [(1 / 3, 1 / 3, 1 / 3, 1 / 3)]
        a, b = rng.dirichlet([1, 1, 1], 2)
        starts.append((a[1], a[2], b[1], b[2]))
        c1, c2 = corners[k % len(corners)], corners[(3 * k + 1) % len(corners)]
        starts.append((c1[0], c1[1], c2[0], c2[1]))
        for x0 in starts:
            x = np.array(x0, dtype=np.float64)
            d2 = ctypes.c_double()
            dc = np.zeros(3)
            ia, na, ta = _lib_patch(patches, tabs, e1)
            ib, nb, tb = _lib_patch(patches, tabs, e2)
            it = harness.lib_smooth_closest(pos.ctypes.data, ia, na, ta, ib, nb, tb, x.ctypes.data,
                                            ctypes.byref(d2), dc.ctypes.data)
            xo, d2o, dco, ito = o.smooth_closest(e1, e2, x0)
            assert np.array_equal(x.view(np.uint64), xo.view(np.uint64)), (e1, e2, x0)
            assert np.float64(d2.value).view(np.uint64) == np.float64(d2o).view(np.uint64)
            assert np.array_equal(dc.view(np.uint64), dco.view(np.uint64))
            assert it == ito
            n_checked += 1
            n_irr += (e1 in irregular) or (e2 in irregular)
    assert n_checked > 150 and n_irr > 50
