"""FP32 element-force path (precision = SHL_PREC_FP32) against the FP64 oracle.

The FP32 path builds strains from the displacement relative to the reference
geometry, so its error is relative to the size of the strains (no metric
cancellation): forces within 1e-4 relative (2-norm) of FP64 at smooth states
with strains of 1e-3 .. 1e-2, exactly zero internal force at the reference
state, and 64-step trajectories within 1e-4 relative of the FP64 oracle.
"""
import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import cell_size_mult_for, classical_pressure, physics_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def smooth_state(X, rng, amp):
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    u = np.stack([amp * x * y, amp * (z * z - 0.3), amp * np.sin(2 * x) * y], 1)
    return (u + 1e-2 * amp * rng.standard_normal(X.shape)).reshape(-1)


@pytest.mark.parametrize("level", [3, 5])
@pytest.mark.parametrize("amp", [1e-3, 2e-2])
def test_fp32_forces_close_to_fp64(cuda_ok, level, amp):
    X, T = L.icosphere(level)
    rng = np.random.default_rng(level)
    p32 = physics_params(contact=False, precision=L.PREC_FP32)
    p64 = physics_params(contact=False)
    g = L.Shell(X, T, p32)
    o = O.Oracle(X, T, p64, threads=4)
    u = smooth_state(X, rng, amp)
    v = np.zeros_like(u)
    for pres in (0.0, -classical_pressure()):
        fg, ag, eg, _ = g.eval_forces(u, v, pres)
        fo, ao, eo, _ = o.eval_forces(u, v, pres)
        assert rel(fg, fo) < 1e-4, (pres, rel(fg, fo))
        for k in ("Etens", "Ebend"):
            assert abs(eg[k] - eo[k]) <= 1e-4 * abs(eo[k]), k
        assert abs(eg["area"] - eo["area"]) <= 1e-6 * eo["area"]


def test_fp32_reference_state_has_no_internal_force(cuda_ok):
    X, T = L.icosphere(4)
    g = L.Shell(X, T, physics_params(contact=False, precision=L.PREC_FP32))
    z = np.zeros(3 * len(X))
    f, _, e, _ = g.eval_forces(z, z, 0.0)
    assert np.all(f == 0.0) and e["Etens"] == 0.0 and e["Ebend"] == 0.0


def test_fp32_trajectory(cuda_ok):
    X, T = L.icosphere(3)
    p64 = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
    p32 = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01), precision=L.PREC_FP32)
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 0).reshape(-1)
    n = 64
    pres = -200 * classical_pressure() * np.arange(1, n + 1) * 1e-4
    g = L.Shell(X, T, p32)
    o = O.Oracle(X, T, p64, threads=4)
    g.apply_initial_conditions(u0, 0.0, pres[0])
    o.apply_initial_conditions(u0, 0.0, pres[0])
    rg, _ = g.step(n, pres)
    ro, _ = o.step(n, pres)
    ug, vg, _ = g.get_state()
    uo, vo, _ = o.get_state()
    assert rel(ug - u0, uo - u0) < 1e-4
    assert rel(vg, vo) < 1e-4
    assert abs(rg.last.Etens - ro.last.Etens) <= 1e-4 * ro.last.Etens
