"""Pressure given as a config expression of t, compiled by the host and
evaluated by the device each step (shl_set_pressure_function): the device
values equal the host evaluation to a few ulp (the device's libm), and a run
with the function equals a run with the same values in the per-step table."""
import math

import numpy as np
import pytest

from shell_gb300 import lib as L
from tests.common import classical_pressure, physics_params

pytestmark = pytest.mark.gpu

EXPR = "-(t < 0.002 ? 1e-4*t/0.002 : 1e-4) * (1 + 0.1*sin(2*pi*t/0.003)) + max(0, 1e-6*log(1+t))"


def host(t):
    ramp = 1e-4 * t / 0.002 if t < 0.002 else 1e-4
    return -ramp * (1 + 0.1 * math.sin(2 * math.pi * t / 0.003)) + max(0.0, 1e-6 * math.log(1 + t))


def test_device_expression_matches_host(cuda_ok):
    X, T = L.icosphere(3)
    g = L.Shell(X, T, physics_params(contact=False))
    g.set_pressure_function(EXPR)
    t = np.linspace(0, 0.01, 257)
    d = g.eval_pressure_function(t)
    h = np.array([host(x) for x in t])
    assert np.all(np.abs(d - h) <= 4e-16 * np.abs(h).max())
    with pytest.raises(L.ShlError):
        g.set_pressure_function("1 + * t")
    with pytest.raises(L.ShlError):
        g.set_pressure_function("x + t")


def test_steps_with_function_equal_table(cuda_ok):
    X, T = L.icosphere(3)
    p = physics_params(contact=True)
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 0).reshape(-1)
    a, b = L.Shell(X, T, p), L.Shell(X, T, p)
    for s in (a, b):
        s.apply_initial_conditions(u0, 0.0, host(p.dt))
    n = 40
    t = np.cumsum(np.full(n, p.dt))
    a.set_pressure_function(EXPR)
    table = a.eval_pressure_function(t)  # the device values, so both runs see the same pressures
    a.step(n, None)
    b.step(n, table)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)
