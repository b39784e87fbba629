"""Adaptive time stepping (ShellSystem.C:1010-1044, 1104-1117) on the GPU
against the CPU oracle: the same accepted steps, the same repeated attempts,
the same dt sequence to 1e-9 (the step-size control feeds the ulp
differences of pow(x, 1/3) on the two libms back into dt), states within
1e-8; the device stopping criterion; the device pressure function with
adaptive steps."""
import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import cell_size_mult_for, classical_pressure, physics_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def mesh3(built):
    return L.icosphere(3)


@pytest.mark.parametrize("dt0,every,contact", [(5e-2, 1, False), (1e-6, 1, False), (2e-2, 3, False),
                                               (1e-3, 1, True)])
def test_adaptive_matches_oracle(cuda_ok, mesh3, dt0, every, contact):
    X, T = mesh3
    p = physics_params(contact=contact, dt=dt0, adapt_dt_every=every, rel_loc_err_min=5e-5, rel_loc_err_max=5e-4,
                       cell_size_mult=cell_size_mult_for(X, T, 0.01))
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 0).reshape(-1)
    g, o = L.Shell(X, T, p), O.Oracle(X, T, p, threads=4)
    pres = -20 * classical_pressure()
    for s in (g, o):
        s.apply_initial_conditions(u0, 0.0, pres)
    n = 40
    rg, sg = g.step(n, np.full(n, pres))
    ro, so = o.step(n, np.full(n, pres))
    assert sg == so and rg.steps_done == ro.steps_done == n
    assert rg.rejections == ro.rejections
    if dt0 == 5e-2:
        assert rg.rejections > 0
    # the step-size control feeds pow(x, 1/3) of the two libms back into dt: agreement to 1e-9
    assert abs(rg.time - ro.time) <= 1e-9 * ro.time
    assert abs(g.dt()[0] - o.dt()) <= 1e-9 * o.dt()
    assert abs(rg.sum_dt - ro.sum_dt) <= 1e-9 * ro.sum_dt
    ug, vg, ag = g.get_state()
    uo, vo, ao = o.get_state()
    assert rel(ug, uo) < 1e-8 and rel(vg, vo) < 1e-7
    if contact:
        assert np.array_equal(g.contact_state()["pairs"], o.contact_state()["pairs"])


def test_adaptive_with_device_pressure_function(cuda_ok, mesh3):
    X, T = mesh3
    p = physics_params(contact=False, dt=1e-2, adapt_dt_every=1, rel_loc_err_min=5e-5, rel_loc_err_max=5e-4)
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 0).reshape(-1)
    expr = "-%r * min(1, t / 0.2)" % float(10 * classical_pressure())
    g, o = L.Shell(X, T, p), O.Oracle(X, T, p, threads=4)
    g.set_pressure_function(expr)
    o.set_pressure_function(expr)
    for s in (g, o):
        s.apply_initial_conditions(u0, 0.0, 0.0)
    rg, _ = g.step(30, None)
    ro, _ = o.step(30, None)
    assert rg.rejections == ro.rejections
    assert abs(rg.time - ro.time) <= 1e-9 * ro.time
    assert rel(g.get_state()[0], o.get_state()[0]) < 1e-8


def test_stop_function(cuda_ok, mesh3):
    X, T = mesh3
    p = physics_params(contact=False, dt=1e-2)
    g = L.Shell(X, T, p)
    g.apply_initial_conditions(np.zeros(X.size), 0.0, 0.0)
    g.set_stop_function("t > 0.35")
    r, st = g.step(100, np.zeros(100))
    t = 0.0
    k = 0
    while not t > 0.35:
        t += 1e-2
        k += 1
    assert r.stopped == 1 and r.steps_done == k and r.time == t
    g.set_stop_function(None)
    r, st = g.step(5, np.zeros(5))
    assert r.stopped == 0 and r.steps_done == 5
