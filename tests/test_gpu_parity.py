"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Tolerances: forces, accelerations and energies of one evaluation within 1e-12
relative (2-norm of the difference over the 2-norm of the oracle vector), the
contact candidate list bit-exact (same pairs, same FP64 squared distances),
friction stick flags identical, spring origins within 1e-12 relative (they
depend on element areas computed by the fused-multiply-add element kernel).  Trajectories agree to 1e-9 relative after
tens of steps (roundoff of the element kernel's fused multiply-adds grows
slowly in time); run-to-run the GPU is bitwise deterministic.
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


def smooth_state(X, rng, amp=0.02):
    """Smooth large displacement plus noise (no contact)."""
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    u = np.stack([amp * x * y, amp * (z * z - 0.3), amp * np.sin(2 * x) * y], 1)
    u += 1e-4 * rng.standard_normal(X.shape)
    return u.reshape(-1)


def squashed_state(X, rng, s=0.0042):
    """The sphere flattened to a double layer of gap about 2*s*|z| (self-contact)."""
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    u += 2e-5 * rng.standard_normal(X.shape)
    return u.reshape(-1)


@pytest.fixture(scope="module")
def meshes(built):
    return {lv: L.icosphere(lv) for lv in (3, 4)}


@pytest.mark.parametrize("level", [3, 4])
@pytest.mark.parametrize("pressure_base", [L.CS_LOCAL, L.CS_SPHERICAL, L.CS_CYLINDRICAL, L.CS_CARTESIAN])
def test_eval_forces_no_contact(cuda_ok, meshes, level, pressure_base):
    X, T = meshes[level]
    rng = np.random.default_rng(level)
    p = physics_params(contact=False, pressure_base=pressure_base, pressure_dir=1, bulk_modulus=0.0)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=4)
    u = smooth_state(X, rng)
    v = 1e-3 * rng.standard_normal(u.shape)
    pres = -classical_pressure()
    fg, ag, eg, sg = g.eval_forces(u, v, pres)
    fo, ao, eo, so = o.eval_forces(u, v, pres)
    assert sg == so == 0
    assert rel(fg, fo) < FORCE_TOL
    assert rel(ag, ao) < FORCE_TOL
    for k in ("Etens", "Ebend", "area"):
        assert abs(eg[k] - eo[k]) <= FORCE_TOL * abs(eo[k]), k
    # per-element fields of the evaluation (curvatures belong to the step's measurement)
    fe_g, fe_o = g.element_fields(), o.element_fields()
    for k in ("etens", "ebend", "area"):
        assert rel(fe_g[k], fe_o[k]) < 1e-11, k
    g.close()


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_FP32])
def test_eval_forces_valence_5_6_7(cuda_ok, precision):
    """A mesh with valence-7 vertices (13-node patches, more than the 12 slots
    of a regular patch): forces and energies against the oracle."""
    X, T = flipped_sphere(1)
    rng = np.random.default_rng(11)
    p = physics_params(contact=False, precision=precision)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, physics_params(contact=False), threads=4)
    u = smooth_state(X, rng)
    v = 1e-3 * rng.standard_normal(u.shape)
    pres = -classical_pressure()
    fg, ag, eg, _ = g.eval_forces(u, v, pres)
    fo, ao, eo, _ = o.eval_forces(u, v, pres)
    tol = FORCE_TOL if precision == L.PREC_FP64 else 1e-4  # FP32: relative to the strain size
    assert rel(fg, fo) < tol
    assert rel(ag, ao) < tol
    for k in ("Etens", "Ebend", "area"):
        assert abs(eg[k] - eo[k]) <= tol * abs(eo[k]), k
    g.close()


@pytest.mark.parametrize("variant", [6, 7, 8, 9, 10])
def test_double_float_variants_match_oracle(cuda_ok, variant):
    """Every launch shape of the double-float element kernel, forced, on a mesh
    with valence-5, -6 and -7 patches (the one-round shape takes faces of all
    patch groups in one block): forces and element fields within 1e-12."""
    X, T = flipped_sphere(1)
    rng = np.random.default_rng(21)
    p = physics_params(contact=False)
    g = L.Shell(X, T, p)
    g.set_element_variant(variant)
    assert g.element_variant()[0] == variant
    o = O.Oracle(X, T, p, threads=4)
    u = smooth_state(X, rng)
    v = 1e-3 * rng.standard_normal(u.shape)
    pres = -classical_pressure()
    fg, ag, eg, _ = g.eval_forces(u, v, pres)
    fo, ao, eo, _ = o.eval_forces(u, v, pres)
    assert rel(fg, fo) < FORCE_TOL and rel(ag, ao) < FORCE_TOL
    fe_g, fe_o = g.element_fields(), o.element_fields()
    for k in ("etens", "ebend", "area"):
        assert rel(fe_g[k], fe_o[k]) < 1e-11, k
    g.close()


def test_mass_damping_match(cuda_ok, meshes):
    X, T = meshes[3]
    p = physics_params(damping_beta=0.01, damping_gamma=0.002)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p)
    Mg, Cg = g.mass_damping()
    Mo, Co = o.mass_damping()
    assert rel(Mg, Mo) < 1e-13
    assert rel(Cg, Co) < 1e-13


@pytest.mark.parametrize("level", [3, 4])
def test_eval_forces_contact_pairs_bitexact(cuda_ok, meshes, level):
    X, T = meshes[level]
    rng = np.random.default_rng(10 + level)
    h = 0.01
    p = physics_params(cell_size_mult=cell_size_mult_for(X, T, h), self_damping=0.01, self_friction_damping=0.01)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=4)
    u = squashed_state(X, rng)
    v = 0.02 * rng.standard_normal(u.shape)
    g.set_state(u, v, np.zeros_like(u))
    o.set_state(u, v, np.zeros_like(u))
    pres = -classical_pressure()
    fg, ag, eg, sg = g.eval_forces(u, v, pres)
    fo, ao, eo, so = o.eval_forces(u, v, pres)
    cg, co = g.contact_state(), o.contact_state()
    assert len(co["pairs"]) > 50, "the squashed state must produce contact candidates"
    assert np.array_equal(cg["pairs"], co["pairs"])
    assert np.array_equal(cg["d2"].view(np.uint64), co["d2"].view(np.uint64))
    assert np.array_equal(cg["stick"], co["stick"])
    assert cg["stick"].sum() > 0
    # spring origins depend on the contact stiffness, which uses the element
    # areas of the (FMA-contracted) element kernel: equal to roundoff
    assert rel(cg["origin"], co["origin"]) < FORCE_TOL
    assert eg["Nc"] == eo["Nc"] and eg["Nc"] > 0
    assert sg == so
    assert rel(fg, fo) < FORCE_TOL
    assert rel(ag, ao) < FORCE_TOL
    assert abs(eg["Eself"] - eo["Eself"]) <= 1e-12 * abs(eo["Eself"])
    assert abs(eg["Efric"] - eo["Efric"]) <= 1e-12 * max(abs(eo["Efric"]), 1e-300)


def test_contact_history_bitexact(cuda_ok, meshes):
    """Kept pairs, sticking pairs and the rebuild from a carried-over list."""
    X, T = meshes[3]
    rng = np.random.default_rng(7)
    p = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=2)
    u = squashed_state(X, rng)
    v = 1e-4 * rng.standard_normal(u.shape)
    for s in (g, o):
        s.set_state(u, v, np.zeros_like(u))
        s.eval_forces(u, v, 0.0)
    c0 = o.contact_state()
    # perturb the list: mark some pairs sticking with origins, make some far
    k = len(c0["pairs"])
    stick = (rng.random(k) < 0.3).astype(np.uint8)
    origin = rng.standard_normal((k, 3)) * stick[:, None]
    d2 = c0["d2"] * np.where(rng.random(k) < 0.3, 100.0, 1.0)
    # a displaced state that needs a rebuild (du_sum above the tolerance)
    u2 = u + 2e-3 * rng.standard_normal(u.shape)
    for s in (g, o):
        s.set_contact_state(c0["pairs"], stick, origin, d2, du_sum=1.0)
        s.set_state(u2, v, np.zeros_like(u))
    fg, _, eg, _ = g.eval_forces(u2, v, 0.0)
    fo, _, eo, _ = o.eval_forces(u2, v, 0.0)
    cg, co = g.contact_state(), o.contact_state()
    assert np.array_equal(cg["pairs"], co["pairs"])
    assert np.array_equal(cg["stick"], co["stick"])
    assert np.array_equal(cg["d2"].view(np.uint64), co["d2"].view(np.uint64))
    assert cg["du_sum"] == co["du_sum"] == 0.0
    assert rel(fg, fo) < FORCE_TOL


@pytest.mark.parametrize("contact", [False, True])
def test_trajectory(cuda_ok, meshes, contact):
    X, T = meshes[3]
    h = 0.01
    p = physics_params(contact=contact, cell_size_mult=cell_size_mult_for(X, T, h))
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=4)
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 0).reshape(-1)
    n = 64
    pres = -2 * classical_pressure() * (np.arange(1, n + 1) * p.dt) / 2.0 * 100.0  # fast ramp
    assert g.apply_initial_conditions(u0, 0.0, pres[0]) == o.apply_initial_conditions(u0, 0.0, pres[0])
    ua, va, aa = g.get_state()
    ub, vb, ab = o.get_state()
    assert rel(aa, ab) < FORCE_TOL
    rg, sg = g.step(n, pres)
    ro, so = o.step(n, pres)
    assert rg.steps_done == ro.steps_done == n
    assert sg == so
    ua, va, aa = g.get_state()
    ub, vb, ab = o.get_state()
    assert rel(ua, ub) < 1e-11
    assert rel(va, vb) < 1e-9
    assert rel(aa, ab) < 1e-9
    assert abs(rg.time - ro.time) == 0.0
    for k in ("sum_Etens", "sum_Ebend", "sum_Ekin", "sum_volume", "sum_area"):
        assert abs(getattr(rg, k) - getattr(ro, k)) <= 1e-9 * abs(getattr(ro, k)), k
    fe_g, fe_o = g.element_fields(), o.element_fields()
    for k in ("kGauss", "kMean", "etens", "ebend", "area"):
        assert rel(fe_g[k], fe_o[k]) < 1e-9, k
    for k in ("kGauss", "kMean", "Etens", "Ebend", "area", "volume", "Ekin"):
        assert abs(getattr(rg.last, k) - getattr(ro.last, k)) <= 1e-9 * abs(getattr(ro.last, k)), k
    if contact:
        assert np.array_equal(g.contact_state()["pairs"], o.contact_state()["pairs"])


def test_graph_equals_direct_and_deterministic(cuda_ok, meshes):
    X, T = meshes[3]
    p = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 1).reshape(-1)
    pres = np.full(40, -classical_pressure())
    states = []
    for use_graph in (True, False, True):
        g = L.Shell(X, T, p)
        g.apply_initial_conditions(u0, 0.0, pres[0])
        g.step(40, pres, use_graph=use_graph)
        states.append(np.concatenate(g.get_state()))
        g.close()
    assert np.array_equal(states[0].view(np.uint64), states[1].view(np.uint64))
    assert np.array_equal(states[0].view(np.uint64), states[2].view(np.uint64))


def test_compat_zero_pressure(cuda_ok, meshes):
    X, T = meshes[3]
    rng = np.random.default_rng(3)
    u = smooth_state(X, rng)
    z = np.zeros_like(u)
    p0 = physics_params(contact=False)
    p1 = physics_params(contact=False, compat_zero_pressure=1)
    f_ref = L.Shell(X, T, p0).eval_forces(u, z, 0.0)[0]
    f_cmp = L.Shell(X, T, p1).eval_forces(u, z, -5.0)[0]
    assert np.array_equal(f_ref, f_cmp)


def test_problem_not_finite(cuda_ok, meshes):
    """A NaN in the state is reported as NOT_FINITE, as the oracle does."""
    X, T = meshes[3]
    p = physics_params(contact=False)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p)
    u = np.zeros(3 * len(X))
    u[5] = np.nan
    z = np.zeros_like(u)
    for s in (g, o):
        s.set_state(u, z, z)
    rg, sg = g.step(3)
    ro, so = o.step(3)
    assert sg == so == 7
    assert rg.steps_done == ro.steps_done == 1


def test_two_contexts_interleaved(cuda_ok, meshes):
    """Two shells with different meshes alive at once keep their own patch
    tables (no state shared through module globals)."""
    rng = np.random.default_rng(11)
    p = physics_params(contact=False)
    shells = {lv: (L.Shell(*meshes[lv], p), O.Oracle(*meshes[lv], p, threads=2)) for lv in (3, 4)}
    for lv in (4, 3, 4):
        X, T = meshes[lv]
        g, o = shells[lv]
        u = smooth_state(X, rng)
        z = np.zeros_like(u)
        assert rel(g.eval_forces(u, z, -1e-4)[0], o.eval_forces(u, z, -1e-4)[0]) < FORCE_TOL
