"""SMOOTH self-contact on the GPU against the CPU oracle.

The closest-point search between limit surfaces is the library's
shl_smooth.h on the GPU and the oracle's own restatement of the same
projected-Newton method on the CPU, both over the shared limit evaluation
(shl_limit.h) and subdivision tables (shl_subdiv.h) with separately rounded
operations, so the candidate list, the squared distances and the searches'
coordinates are bit-exact at a given state; forces
within 1e-12 relative (the element kernel's fused multiply-adds); 24-step
trajectories within 1e-10 (u) and 1e-7 (v): the searches stop within their
convergence tolerance, which a 1e-13 force difference can shift.
"""
import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import cell_size_mult_for, classical_pressure, flipped_sphere, physics_params

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def squashed_state(X, rng, s=0.0042):
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    u += 2e-5 * rng.standard_normal(X.shape)
    return u.reshape(-1)


def smooth_params(X, T, **kw):
    return physics_params(shell_shell_contact=L.CONTACT_SMOOTH, cell_size_mult=cell_size_mult_for(X, T, 0.01),
                          self_damping=0.01, self_friction_damping=0.01, **kw)


@pytest.fixture(scope="module")
def meshes(built):
    return {"ico3": L.icosphere(3), "flip": flipped_sphere(1)}


@pytest.mark.parametrize("name", ["ico3", "flip"])
def test_smooth_eval_forces_bitexact_pairs(cuda_ok, meshes, name):
    X, T = meshes[name]
    rng = np.random.default_rng(21)
    p = smooth_params(X, T)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=4)
    u = squashed_state(X, rng)
    v = 0.02 * rng.standard_normal(u.shape)
    for s in (g, o):
        s.set_state(u, v, np.zeros_like(u))
    pres = -classical_pressure()
    fg, ag, eg, sg = g.eval_forces(u, v, pres)
    fo, ao, eo, so = o.eval_forces(u, v, pres)
    cg, co = g.contact_state(), o.contact_state()
    assert len(co["pairs"]) > 50
    assert np.array_equal(cg["pairs"], co["pairs"])
    assert np.array_equal(cg["d2"].view(np.uint64), co["d2"].view(np.uint64))
    xg, xo = g.contact_coords(), o.contact_coords()
    assert np.array_equal(xg.view(np.uint64), xo.view(np.uint64))
    assert np.any(np.abs(xg - 1 / 3) > 1e-3)
    assert np.array_equal(cg["stick"], co["stick"])
    assert rel(cg["origin"], co["origin"]) < FORCE_TOL
    assert eg["Nc"] == eo["Nc"] and eg["Nc"] > 0
    assert sg == so
    assert rel(fg, fo) < FORCE_TOL
    assert rel(ag, ao) < FORCE_TOL
    assert abs(eg["Eself"] - eo["Eself"]) <= 1e-12 * abs(eo["Eself"])
    g.close()


def test_smooth_differs_from_linear(cuda_ok, meshes):
    """The limit surfaces lie inside the facets of a convex region: the
    SMOOTH distances of the same pairs differ from the LINEAR ones, and the
    candidate search reaches farther (d_max grows by the mean element size)."""
    X, T = meshes["ico3"]
    rng = np.random.default_rng(22)
    u = squashed_state(X, rng)
    z = np.zeros_like(u)
    lin = L.Shell(X, T, physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01)))
    smo = L.Shell(X, T, smooth_params(X, T))
    for s in (lin, smo):
        s.set_state(u, z, z)
        s.eval_forces(u, z, 0.0)
    cl, cs = lin.contact_state(), smo.contact_state()
    assert len(cs["pairs"]) > len(cl["pairs"])
    common = {tuple(p): d for p, d in zip(cl["pairs"], cl["d2"])}
    diffs = [abs(d - common[tuple(p)]) / common[tuple(p)] for p, d in zip(cs["pairs"], cs["d2"]) if tuple(p) in common]
    assert len(diffs) > 20 and np.median(diffs) > 1e-4


@pytest.mark.parametrize("name", ["ico3", "flip"])
def test_smooth_trajectory(cuda_ok, meshes, name):
    """Steps from a squashed state (contacts, friction, rebuilds) against the oracle."""
    X, T = meshes[name]
    rng = np.random.default_rng(23)
    p = smooth_params(X, T)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=4)
    u = squashed_state(X, rng)
    v = 1e-3 * rng.standard_normal(u.shape)
    for s in (g, o):
        s.set_state(u, v, np.zeros_like(u))
        s.rebuild_contacts()
    n = 24
    pres = np.full(n, -0.5 * classical_pressure())
    rg, sg = g.step(n, pres)
    ro, so = o.step(n, pres)
    assert sg == so and rg.steps_done == ro.steps_done == n
    ua, va, _ = g.get_state()
    ub, vb, _ = o.get_state()
    # the searches stop within their convergence tolerance (Newton decrement
    # 1e-15 f, steps of 1e-6 after a full Newton step), and a 1e-13 difference
    # of the element forces can change where one stops
    assert rel(ua, ub) < 1e-10
    assert rel(va, vb) < 1e-7
    cg, co = g.contact_state(), o.contact_state()
    assert np.array_equal(cg["pairs"], co["pairs"])
    assert np.array_equal(cg["stick"], co["stick"])
    assert np.abs(g.contact_coords() - o.contact_coords()).max() < 1e-5  # search steps stop at 1e-6
    assert abs(rg.sum_Eself - ro.sum_Eself) <= 1e-9 * abs(ro.sum_Eself)
    g.close()


def test_contact_coords_round_trip(cuda_ok, meshes):
    X, T = meshes["ico3"]
    rng = np.random.default_rng(24)
    g = L.Shell(X, T, smooth_params(X, T))
    u = squashed_state(X, rng)
    g.set_state(u, np.zeros_like(u), np.zeros_like(u))
    g.rebuild_contacts()
    x = g.contact_coords()
    assert len(x) > 50
    y = np.clip(x + 0.01, 0, 0.45)
    g.set_contact_coords(y)
    assert np.array_equal(g.contact_coords(), y)
    cs = g.contact_state()
    g.set_contact_state(cs["pairs"], cs["stick"], cs["origin"], cs["d2"])
    assert np.all(g.contact_coords() == 1 / 3)
    g.close()
