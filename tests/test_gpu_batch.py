"""Batched shells (shl_batch_create): a batch advances every shell exactly as
the shell would advance alone (same per-face arithmetic, same per-node
summation order), so states are compared bit for bit."""
import numpy as np
import pytest

from shell_gb300 import lib as L
from tests.common import classical_pressure, physics_params

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


def test_batch_rejects_contact_and_mixed_dt(cuda_ok):
    X, T = L.icosphere(3)
    with pytest.raises(L.ShlError):
        L.Batch([(X, T), (X, T)], [physics_params(contact=True), physics_params(contact=True)])
    with pytest.raises(L.ShlError):
        L.Batch([(X, T), (X, T)], [physics_params(contact=False), physics_params(contact=False, dt=2e-4)])
