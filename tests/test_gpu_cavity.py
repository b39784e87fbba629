"""Cavity contact (ShellSystem.C:1600-1723) on the GPU against the CPU oracle:
one force evaluation per cavity shape (box, cylinder, ellipsoid) with friction
and normal damping -- forces within 1e-12 relative, spring origins and
per-node energy densities within 1e-12 -- and a trajectory inside a shrinking
ellipsoid given as a device-evaluated expression of t (1e-10)."""
import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import physics_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def cavity_params(kind, **kw):
    base = dict(contact=False, shell_cavity_contact=1, cavity=kind, Rx=1.004, Ry=0.98, Rz=1.001, mu_s_cavity=0.4,
                mu_d_cavity=0.3, cavity_damping=0.01, cavity_friction_damping=0.01)
    base.update(kw)
    return physics_params(**base)


@pytest.mark.parametrize("kind", [L.CAVITY_BOX, L.CAVITY_CYLINDER, L.CAVITY_ELLIPSOID])
def test_cavity_forces_match_oracle(cuda_ok, kind):
    X, T = L.icosphere(3)
    p = cavity_params(kind) if kind != L.CAVITY_BOX else cavity_params(kind, Rx=0.985, Ry=1.2, Rz=0.99)
    rng = np.random.default_rng(kind)
    u = 2e-3 * rng.standard_normal(X.size)
    v = 0.05 * rng.standard_normal(X.size)
    g, o = L.Shell(X, T, p), O.Oracle(X, T, p, threads=4)
    for s in (g, o):
        s.set_state(u, v, np.zeros_like(u))
    fg, ag, eg, _ = g.eval_forces(u, v, -1e-4)
    fo, ao, eo, _ = o.eval_forces(u, v, -1e-4)
    co = o.cavity()
    assert co["Nc_cav"] > 10
    assert rel(fg, fo) < 1e-12
    assert rel(g.cavity_origins(), co["origins"]) < 1e-12
    assert np.count_nonzero(co["origins"]) > 0


def test_cavity_trajectory_shrinking_ellipsoid(cuda_ok):
    X, T = L.icosphere(3)
    p = cavity_params(L.CAVITY_ELLIPSOID, Rx=1.01, Ry=1.01, Rz=1.01, damping_alpha=0.5, dt=1e-3)
    expr = ["1.01 - 0.5*t", "1.01 - 0.4*t", "1.01 - 0.6*t"]
    g, o = L.Shell(X, T, p), O.Oracle(X, T, p, threads=4)
    g.set_cavity_functions(*expr)
    o.set_cavity_functions(*expr)
    u0 = L.gaussian_normal_imperfection(X, 1e-4, 0).reshape(-1)
    for s in (g, o):
        s.apply_initial_conditions(u0, 0.0, 0.0)
    n = 60
    rg, sg = g.step(n, np.zeros(n))
    ro, so = o.step(n, np.zeros(n))
    assert sg == so and rg.steps_done == ro.steps_done == n
    assert rg.last.Nc_cav == ro.last.Nc_cav and ro.last.Nc_cav > 0
    for k in ("sum_pcav", "sum_Nc_cav", "sum_Ecav", "sum_Efric", "sum_Ekin"):
        assert abs(getattr(rg, k) - getattr(ro, k)) <= 1e-9 * abs(getattr(ro, k)), k
    assert rel(g.get_state()[0], o.get_state()[0]) < 1e-10
    nf = g.node_fields()
    assert rel(nf["ecav"], o.cavity()["ecav"]) < 1e-9
    assert rel(nf["efric"], o.node_fields()["efric"]) < 1e-9
