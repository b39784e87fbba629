"""Batched shells (shl_batch_create): a batch advances every shell exactly as
the shell would advance alone (same per-face arithmetic, same per-node
summation order), so states are compared bit for bit."""
import numpy as np
import pytest

from shell_gb300 import lib as L
from tests.common import cell_size_mult_for, classical_pressure, physics_params

pytestmark = pytest.mark.gpu


def _shells():
    specs = [(3, dict(thickness=0.01)), (4, dict(thickness=0.02, shell_young_modulus2=2.0)),
             (3, dict(thickness=0.005, shell_young_modulus=3.0, damping_alpha=0.2))]
    out = []
    for lv, kw in specs:
        X, T = L.icosphere(lv)
        out.append((X, T, kw))
    return out


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_FP32])
def test_batch_equals_single_shells(cuda_ok, precision):
    shells = _shells()
    scales = np.array([1.0, 2.5, 0.7])
    params = [physics_params(contact=False, precision=precision, **kw) for _, _, kw in shells]
    b = L.Batch([(X, T) for X, T, _ in shells], params, pressure_scale=scales)
    assert b.n_shells == 3 and b.F == sum(len(T) for _, T, _ in shells)
    u0s = [L.gaussian_normal_imperfection(X, 1e-3, k).reshape(-1) for k, (X, _, _) in enumerate(shells)]
    n = 24
    pres = -50 * classical_pressure() * np.arange(1, n + 1) * 1e-4
    b.apply_initial_conditions(np.concatenate(u0s), 0.0, pres[0])
    rb, sb = b.step(n, pres)
    assert sb == 0 and rb.steps_done == n
    ub, vb, ab = b.get_state()
    for k, (X, T, kw) in enumerate(shells):
        g = L.Shell(X, T, params[k])
        g.apply_initial_conditions(u0s[k], 0.0, pres[0] * scales[k])
        g.step(n, pres * scales[k])
        u, v, a = g.get_state()
        for x, y in ((u, b.split(ub)[k]), (v, b.split(vb)[k]), (a, b.split(ab)[k])):
            assert np.array_equal(x.view(np.uint64), np.ascontiguousarray(y).view(np.uint64))
        g.close()


def test_batch_rejects_mixed_contact_and_dt(cuda_ok):
    X, T = L.icosphere(3)
    with pytest.raises(L.ShlError):  # self-contact on in one shell only
        L.Batch([(X, T), (X, T)], [physics_params(contact=True), physics_params(contact=False)])
    with pytest.raises(L.ShlError):  # different friction coefficients
        L.Batch([(X, T), (X, T)], [physics_params(contact=True), physics_params(contact=True, mu_s=0.5)])
    with pytest.raises(L.ShlError):  # self-contact with adaptive dt
        L.Batch([(X, T), (X, T)], [physics_params(contact=True, adapt_dt_every=10, rel_loc_err_min=5e-5,
                                                  rel_loc_err_max=5e-4)] * 2)
    with pytest.raises(L.ShlError):
        L.Batch([(X, T), (X, T)], [physics_params(contact=False), physics_params(contact=False, dt=2e-4)])


def _squashed(X, seed, s=0.0042):
    """The sphere flattened to a double layer with seeded noise: every face has
    contact candidates on the other layer and the lists are rebuilt as it moves."""
    rng = np.random.default_rng(seed)
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    return (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_self_contact_equals_single_shells(cuda_ok, use_graph):
    """Each shell of a batch keeps its own linked cells (trigger, bounds, cell
    size, d_max, grid), so state, candidate list, friction state, du_sum and
    rebuild count equal those of the shell run alone, bit for bit."""
    specs = [(3, 0.01, {}, 3), (4, 0.01, dict(shell_young_modulus2=2.0), 4),
             (3, 0.015, dict(shell_young_modulus=3.0, damping_alpha=0.2), 5)]
    meshes, params, u0s = [], [], []
    for lv, h, kw, seed in specs:
        X, T = L.icosphere(lv)
        meshes.append((X, T))
        params.append(physics_params(thickness=h, cell_size_mult=cell_size_mult_for(X, T, h), **kw))
        u0s.append(_squashed(X, seed))
    n = 24
    table = np.zeros(n)
    b = L.Batch(meshes, params)
    z = np.zeros(3 * b.V)
    b.set_state(np.concatenate(u0s), z, z)
    b.rebuild_contacts()
    rb, sb = b.step(n, table, use_graph=use_graph)
    assert rb.steps_done == n
    ub, vb, ab = b.get_state()
    cb = b.contact_state()
    du_b, nr_b = b.contact_stats()
    pairs_b = b.split_pairs(cb["pairs"])
    shell_of_pair = np.searchsorted(b.face_off, cb["pairs"].reshape(-1, 2)[:, 0], side="right") - 1
    b.close()
    for k, ((X, T), p, u0) in enumerate(zip(meshes, params, u0s)):
        g = L.Shell(X, T, p)
        zz = np.zeros_like(u0)
        g.set_state(u0, zz, zz)
        g.rebuild_contacts()
        rg, sg = g.step(n, table, use_graph=use_graph)
        u, v, a = g.get_state()
        for x, y in ((u, b.split(ub)[k]), (v, b.split(vb)[k]), (a, b.split(ab)[k])):
            assert np.array_equal(_bits(x), _bits(y))
        c = g.contact_state()
        assert len(c["pairs"]) > 0, "the squashed shell is in contact"
        assert np.array_equal(np.asarray(c["pairs"]).reshape(-1, 2), pairs_b[k])
        sel = shell_of_pair == k
        assert np.array_equal(c["stick"], cb["stick"][sel])
        assert np.array_equal(_bits(c["origin"]), _bits(cb["origin"][sel]))
        assert np.array_equal(_bits(c["d2"]), _bits(cb["d2"][sel]))
        assert c["du_sum"] == du_b[k]
        assert rg.n_rebuilds >= 1 and nr_b[k] == rg.n_rebuilds + 1  # + the rebuild before the steps
        g.close()


def test_batch_smooth_contact_equals_single_shells(cuda_ok):
    """SMOOTH self-contact in a batch: the limit patches (valence tables, patch
    frames) and the closest-point searches of each shell equal those of the
    shell run alone, bit for bit (pairs, d2, search coordinates, state)."""
    specs = [(3, 0.01, {}, 3), (3, 0.015, dict(shell_young_modulus2=2.0), 5)]
    meshes, params, u0s = [], [], []
    for lv, h, kw, seed in specs:
        X, T = L.icosphere(lv)
        meshes.append((X, T))
        params.append(physics_params(thickness=h, cell_size_mult=cell_size_mult_for(X, T, h),
                                     shell_shell_contact=L.CONTACT_SMOOTH, **kw))
        u0s.append(_squashed(X, seed))
    n = 8
    table = np.zeros(n)
    b = L.Batch(meshes, params)
    z = np.zeros(3 * b.V)
    b.set_state(np.concatenate(u0s), z, z)
    b.rebuild_contacts()
    rb, sb = b.step(n, table)
    assert rb.steps_done == n
    ub, vb, ab = b.get_state()
    cb = b.contact_state()
    xb = b.contact_coords()
    pairs_b = b.split_pairs(cb["pairs"])
    shell_of_pair = np.searchsorted(b.face_off, cb["pairs"].reshape(-1, 2)[:, 0], side="right") - 1
    b.close()
    for k, ((X, T), p, u0) in enumerate(zip(meshes, params, u0s)):
        g = L.Shell(X, T, p)
        zz = np.zeros_like(u0)
        g.set_state(u0, zz, zz)
        g.rebuild_contacts()
        g.step(n, table)
        u, v, a = g.get_state()
        for x, y in ((u, b.split(ub)[k]), (v, b.split(vb)[k]), (a, b.split(ab)[k])):
            assert np.array_equal(_bits(x), _bits(y))
        c = g.contact_state()
        assert len(c["pairs"]) > 0, "the squashed shell is in contact"
        assert np.array_equal(np.asarray(c["pairs"]).reshape(-1, 2), pairs_b[k])
        sel = shell_of_pair == k
        assert np.array_equal(_bits(c["d2"]), _bits(cb["d2"][sel]))
        assert np.array_equal(_bits(g.contact_coords()), _bits(xb[sel]))
        g.close()
