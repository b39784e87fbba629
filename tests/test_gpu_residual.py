"""Relative residual ||f_ext - f_int|| / ||f_ext|| (shl_residual), single shells
and batches, against the CPU oracle: f from an oracle force evaluation
without self-contact, f_ext from one with the stiffness multipliers set to 0,
both without their rigid-translation part (resultant spread by nodal mass).
Tolerance 1e-10 relative on the residual in FP64 (norms of 1e-12-accurate
vectors); in FP32 the residual of an equilibrium is only resolved down to the
FP32 force error (about 1e-6 of the force scale)."""
import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import classical_pressure, physics_params

pytestmark = pytest.mark.gpu


def _oracle_residual(X, T, p, u, pressure):
    o = O.Oracle(X, T, p, threads=4)
    o.set_state(u, np.zeros_like(u), np.zeros_like(u))
    f = o.eval_forces(u, np.zeros_like(u), pressure)[0]
    q = L.default_params(**{k: getattr(p, k) for k, _ in L.ShlParams._fields_})
    q.memb_stiff_mult = 0.0
    q.bend_stiff_mult = 0.0
    o2 = O.Oracle(X, T, q, threads=4)
    o2.set_state(u, np.zeros_like(u), np.zeros_like(u))
    fe = o2.eval_forces(u, np.zeros_like(u), pressure)[0]
    m = 1.0 / o.mass_damping()[0].reshape(-1, 3)[:, :1]

    def drop_translation(x):  # the resultant spread over the nodes by mass
        x = x.reshape(-1, 3)
        return (x - m * (x.sum(0) / m.sum())).reshape(-1)

    f, fe = drop_translation(f), drop_translation(fe)
    return np.linalg.norm(f) / np.linalg.norm(fe), f, fe


def test_residual_single_matches_oracle(cuda_ok):
    X, T = L.icosphere(3)
    rng = np.random.default_rng(4)
    p = physics_params(contact=False)
    u = 1e-3 * rng.standard_normal(X.size)
    pres = -classical_pressure()
    g = L.Shell(X, T, p)
    g.set_state(u, np.zeros_like(u), np.zeros_like(u))
    r = g.residual(pres)
    ro, _, _ = _oracle_residual(X, T, p, u, pres)
    assert r.shape == (1,)
    assert abs(r[0] - ro) <= 1e-10 * ro
    # the stored state is untouched and stepping continues normally
    u2, _, _ = g.get_state()
    assert np.array_equal(u2, u)


def test_residual_batch_per_shell(cuda_ok):
    meshes = [L.icosphere(3), L.icosphere(4), L.icosphere(3)]
    rng = np.random.default_rng(5)
    ps = [physics_params(contact=False, thickness=h, shell_young_modulus2=e2)
          for h, e2 in ((0.01, 0.5), (0.02, 1.0), (0.005, 2.0))]
    scale = np.array([1.0, 0.5, 2.0])
    b = L.Batch(meshes, ps, scale)
    us = [1e-3 * rng.standard_normal(X.size) for X, _ in meshes]
    u = np.concatenate(us)
    b.set_state(u, np.zeros_like(u), np.zeros_like(u))
    pres = -classical_pressure()
    r = b.residual(pres)
    for k, ((X, T), p) in enumerate(zip(meshes, ps)):
        ro, _, _ = _oracle_residual(X, T, p, us[k], pres * scale[k])
        assert abs(r[k] - ro) <= 1e-10 * ro, k


def test_residual_fp64_in_fp32_context_and_defect_correction(cuda_ok):
    """An FP32 batch evaluates its residual with FP64 forces on request (the
    same value as an FP64 batch at the same state); with the defect correction
    its relaxation reaches the FP64 residual tolerance and the FP64
    equilibrium, which plain FP32 relaxation cannot."""
    meshes = [L.icosphere(3), L.icosphere(3)]
    ps32 = [physics_params(contact=False, damping_alpha=1.5, dt=4e-3, precision=L.PREC_FP32, thickness=h)
            for h in (0.01, 0.02)]
    ps64 = [physics_params(contact=False, damping_alpha=1.5, dt=4e-3, thickness=h) for h in (0.01, 0.02)]
    scale = np.array([0.2 * classical_pressure(h=0.01), 0.2 * classical_pressure(h=0.02)])
    rng = np.random.default_rng(6)
    u = 1e-3 * rng.standard_normal(2 * meshes[0][0].size)
    b32, b64 = L.Batch(meshes, ps32, scale), L.Batch(meshes, ps64, scale)
    for b in (b32, b64):
        b.set_state(u, np.zeros_like(u), np.zeros_like(u))
    r64 = b64.residual(-1.0)
    r32_64 = b32.residual(-1.0, L.RESIDUAL_FP64)
    assert np.allclose(r32_64, r64, rtol=1e-13, atol=0)
    r32 = b32.residual(-1.0)
    assert np.all(np.abs(r32 - r64) <= 1e-3 * r64)

    def relax(b, flags, n_checks=40, every=100):
        b.apply_initial_conditions(np.zeros_like(u), 0.0, -1.0)
        r = b.residual(-1.0, flags)
        for _ in range(n_checks):
            b.step(every, np.full(every, -1.0))
            r = b.residual(-1.0, flags)
        return r, b.get_state()[0]

    # the same 4,000 steps: FP32 relaxation with the FP64 defect follows the FP64 one
    r_ref, u_ref = relax(b64, 0)
    r_c, u_c = relax(b32, L.RESIDUAL_FP64 | L.RESIDUAL_CORRECT)
    assert np.all(np.abs(r_c - r_ref) <= 1e-3 * r_ref + 1e-7)
    assert np.abs(u_c - u_ref).max() < 1e-4 * np.abs(u_ref).max()


def test_residual_with_self_contact_matches_oracle(cuda_ok):
    """SHL_RESIDUAL_CONTACT: the static self-contact force of the current
    candidate list joins f_int (frictionless contact, no contact damping).  At
    rest (v = 0) it equals the oracle's force evaluation with contact at the
    same state; the contact state is left as it was."""
    from tests.common import cell_size_mult_for
    X, T = L.icosphere(3)
    rng = np.random.default_rng(6)
    u = np.zeros_like(X)
    u[:, 2] = (0.0042 - 1.0) * X[:, 2]
    u = (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)
    p = physics_params(mu_s=0.0, mu_d=0.0, cell_size_mult=cell_size_mult_for(X, T, 0.01))
    pres = -classical_pressure()
    z = np.zeros_like(u)
    g = L.Shell(X, T, p)
    g.set_state(u, z, z)
    g.rebuild_contacts()
    before = g.contact_state()
    assert len(before["pairs"]) > 1000
    r_plain = g.residual(pres)
    r = g.residual(pres, L.RESIDUAL_CONTACT)
    after = g.contact_state()
    for k in ("pairs", "stick", "origin", "d2"):
        assert np.array_equal(np.asarray(before[k]), np.asarray(after[k])), k
    o = O.Oracle(X, T, p, threads=4)
    o.set_state(u, z, z)
    o.rebuild_contacts()
    f = o.eval_forces(u, z, pres)[0]
    _, _, fe = _oracle_residual(X, T, physics_params(contact=False), u, pres)
    m = 1.0 / o.mass_damping()[0].reshape(-1, 3)[:, :1]
    x = f.reshape(-1, 3)
    x = (x - m * (x.sum(0) / m.sum())).reshape(-1)
    ro = np.linalg.norm(x) / np.linalg.norm(fe)
    assert abs(r[0] - ro) <= 1e-10 * ro
    assert abs(r[0] - r_plain[0]) > 1e-3 * r_plain[0]  # the contact force matters at this state
    with pytest.raises(L.ShlError):  # friction makes the contact force path dependent
        q = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
        g2 = L.Shell(X, T, q)
        g2.set_state(u, z, z)
        g2.residual(pres, L.RESIDUAL_CONTACT)
    g.close()
