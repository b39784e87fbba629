"""The command-line driver shl_run (csrc/shl_run.cpp): config parsing, the
expression language, command-line overrides, unsupported options, and (on a
GPU) a full run with table, VTU and state-file output and a resume from the
state file, checked bit for bit against the same steps through the Python
binding.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from shell_gb300 import build as B
from shell_gb300 import lib as L

RUN = B.RUN


@pytest.fixture(scope="module")
def driver(built):
    if not os.path.exists(RUN):
        pytest.skip("shl_run not built")
    return RUN


def _write(tmp_path, cfg_text, level=3):
    (tmp_path / "c.cfg").write_text(cfg_text)
    (tmp_path / "m.off").write_text(L.icosphere_off(level))
    return str(tmp_path / "c.cfg"), str(tmp_path / "m.off")


def _run(driver, *args, cwd=None):
    r = subprocess.run([driver, *args], capture_output=True, text=True, cwd=cwd, timeout=600)
    return r.returncode, r.stdout


BASE_CFG = """
# shell
shell_mass_density  = 1
shell_young_modulus = 1
shell_young_modulus2 = 0.5        # E2
shell_poisson_ratio = 0.3
shell_shear_modulus = 0.35
thickness           = 0.01
damping_alpha       = 0.05
dt                  = 1e-4
pressure            = -2*0.001*t/2  # ramp
pressure_base       = local
shell_shell_contact = none
shell_cavity_contact = false
adapt_dt_every      = 0
distortion          = 0.1
random_seed         = 7
"""


def _dry(driver, tmp_path, cfg, *extra):
    c, m = _write(tmp_path, cfg)
    rc, out = _run(driver, "-c", c, "-m", m, "--dry-run", *extra)
    assert rc == 0, out
    return json.loads(out.strip().splitlines()[-1]), out


def test_dry_run_parses_config(driver, tmp_path):
    d, out = _dry(driver, tmp_path, BASE_CFG)
    assert d["nodes"] == 642 and d["faces"] == 1280
    assert d["shell_young_modulus2"] == 0.5 and d["shell_poisson_ratio"] == 0.3
    assert d["pressure_at"] == [-2 * 0.001 * (k * 1e-4) / 2 for k in (1, 2, 3, 4)] or np.allclose(
        d["pressure_at"], [-1e-3 * k * 1e-4 for k in (1, 2, 3, 4)], rtol=1e-15)
    assert d["random_seed"] == 7 and d["distortion"] == 0.1
    assert "WARNING: Parameter time_steps is missing" in out


def test_expressions_and_overrides(driver, tmp_path):
    cfg = BASE_CFG + "shell_poisson_ratio = 1/3\nthickness = 2^-2*0.04\nstopping_criterion = t>0.3 && t<1\n"
    d, _ = _dry(driver, tmp_path, cfg, "-dt", "5e-5", "-pressure", "-(1+sin(pi/2))*t", "-scale", "2,2,2",
                "-shell_young_modulus", "max(3,4,2)")
    assert d["shell_poisson_ratio"] == 1 / 3
    assert d["thickness"] == 0.01
    assert d["dt"] == 5e-5
    assert d["shell_young_modulus"] == 4
    assert np.allclose(d["pressure_at"], [-2 * k * 5e-5 for k in (1, 2, 3, 4)], rtol=1e-14)
    X, _ = L.icosphere(3)
    assert d["x0"] == 2 * X[0, 0] and d["z0"] == 2 * X[0, 2]
    assert d["stop_at_0"] == 0


def test_mesh_transforms(driver, tmp_path):
    X, _ = L.icosphere(3)
    d, _ = _dry(driver, tmp_path, BASE_CFG + "project = 2,2,2\ntranslate = 1,0,-1\n")
    r = np.linalg.norm(X[0])
    assert abs(d["x0"] - (X[0, 0] * 2 / r + 1)) < 1e-15 and abs(d["z0"] - (X[0, 2] * 2 / r - 1)) < 1e-15
    d, _ = _dry(driver, tmp_path, BASE_CFG + "refinements = 1\n")
    assert d["nodes"] == 2562 and d["faces"] == 5120


def test_smooth_contact_accepted(driver, tmp_path):
    d, _ = _dry(driver, tmp_path, BASE_CFG + "shell_shell_contact = smooth\n")
    assert d["shell_shell_contact"] == L.CONTACT_SMOOTH


@pytest.mark.parametrize("bad", ["growth1 = 1.1", "shell_shell_contact = curved",
                                 "thickness = 0.01*(1+t)", "gravity = 9.81", "pressure = 2*", "extra_order = 1"])
def test_unsupported_options_fail(driver, tmp_path, bad):
    c, m = _write(tmp_path, BASE_CFG + bad + "\n")
    rc, out = _run(driver, "-c", c, "-m", m, "--dry-run")
    assert rc == 3 and "ERROR" in out, out


def test_missing_files(driver, tmp_path):
    rc, out = _run(driver, "-c", str(tmp_path / "none.cfg"))
    assert rc == 3 and "Can't open config file" in out
    c, _ = _write(tmp_path, BASE_CFG)
    rc, out = _run(driver, "-c", c, "-m", str(tmp_path / "none.off"), "--dry-run")
    assert rc == 3 and "mesh file" in out


class Drand48:
    """POSIX srand48/drand48: X <- (0x5DEECE66D X + 0xB) mod 2^48, seeded with (seed << 16) | 0x330E."""

    def __init__(self, seed):
        self.x = ((seed & 0xFFFFFFFF) << 16) | 0x330E

    def __call__(self):
        self.x = (0x5DEECE66D * self.x + 0xB) & ((1 << 48) - 1)
        return self.x / float(1 << 48)


@pytest.mark.gpu
def test_run_resume_and_match_binding(driver, cuda_ok, tmp_path):
    cfg = BASE_CFG + "shell_shell_contact = linear\nmu_s = 0.3\nmu_d = 0.3\ncell_size_mult = 1\n" \
                     "data_time = 0.001\nvtk_time = 0.002\nstate_time = 0\ntime_steps = 40\n"
    c, m = _write(tmp_path, cfg)
    d1 = str(tmp_path / "d1")
    rc, out = _run(driver, "-c", c, "-m", m, "-d", d1)
    assert rc == 0, out
    # outputs when int(t / interval) grows, t accumulated step by step as the reference does
    t, data_steps, vtk_steps = 0.0, [], [0]
    for k in range(1, 41):
        t_new = t + 1e-4
        if int(t_new / 0.001) > int(t / 0.001):
            data_steps.append(k)
        if int(t_new / 0.002) > int(t / 0.002):
            vtk_steps.append(k)
        t = t_new
    table = [ln for ln in out.splitlines() if ln.startswith("# ")]
    assert len(table) == 1 + len(data_steps)
    assert [int(ln.split()[2]) for ln in table] == [0] + data_steps
    assert sorted(os.listdir(d1)) == sorted(["c.cfg", "m.off", "shell_state0000000040.dat", "shell_state_latest.dat"] +
                                            ["shell%010d.vtu" % k for k in vtk_steps])
    # the same run through the binding: drand48 distortion, per-step pressure table
    X, T = L.icosphere(3)
    p = L.default_params(shell_mass_density=1.0, shell_young_modulus=1.0, shell_young_modulus2=0.5,
                         shell_poisson_ratio=0.3, shell_shear_modulus=0.35, thickness=0.01, damping_alpha=0.05,
                         dt=1e-4, shell_shell_contact=L.CONTACT_LINEAR, mu_s=0.3, mu_d=0.3, cell_size_mult=1.0)
    rng = Drand48(7)
    u0 = np.array([0.1 * (2 * rng() - 1) * 0.01 for _ in range(3 * X.shape[0])])
    g = L.Shell(X, T, p)
    ts = np.cumsum(np.full(41, 1e-4))
    g.apply_initial_conditions(u0, 0.0, -2 * 0.001 * ts[0] / 2)
    for k in range(4):
        g.step(10, -2 * 0.001 * ts[10 * k:10 * k + 10] / 2)
    u_bind = g.get_state()
    g2 = L.Shell(X, T, p)
    g2.load_state_file(os.path.join(d1, "shell_state0000000040.dat"))
    for x, y in zip(u_bind, g2.get_state()):
        assert np.array_equal(x, y)
    # resume for 20 more steps from the state file
    d2 = str(tmp_path / "d2")
    os.makedirs(d2)
    rc, out = _run(driver, "-c", c, "-m", m, "-d", d2, "-l", os.path.join(d1, "shell_state_latest.dat"),
                   "-time_steps", "60")
    assert rc == 0, out
    assert os.path.exists(os.path.join(d2, "shell_state0000000060.dat"))
    for k in range(4, 6):
        g.step(10, -2 * 0.001 * np.cumsum(np.full(60, 1e-4))[10 * k:10 * k + 10] / 2)
    g3 = L.Shell(X, T, p)
    step, dt, _, rows = g3.load_state_file(os.path.join(d2, "shell_state0000000060.dat"))
    assert step == 60 and dt == 1e-4
    for x, y in zip(g.get_state(), g3.get_state()):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_run_adaptive_dt_matches_binding(driver, cuda_ok, tmp_path):
    cfg = BASE_CFG + "adapt_dt_every = 1\ndt = 2e-2\nrel_loc_err_min = 5e-5\nrel_loc_err_max = 5e-4\n" \
                     "pressure = -1e-3*min(1, t/0.5)\ndata_time = 0.05\nvtk_time = 0\nstate_time = 0\ntime_steps = 30\n"
    c, m = _write(tmp_path, cfg)
    d1 = str(tmp_path / "d1")
    rc, out = _run(driver, "-c", c, "-m", m, "-d", d1)
    assert rc == 0, out
    X, T = L.icosphere(3)
    p = L.default_params(shell_mass_density=1.0, shell_young_modulus=1.0, shell_young_modulus2=0.5,
                         shell_poisson_ratio=0.3, shell_shear_modulus=0.35, thickness=0.01, damping_alpha=0.05,
                         dt=2e-2, shell_shell_contact=L.CONTACT_NONE, adapt_dt_every=1, rel_loc_err_min=5e-5,
                         rel_loc_err_max=5e-4)
    rng = Drand48(7)
    u0 = np.array([0.1 * (2 * rng() - 1) * 0.01 for _ in range(3 * X.shape[0])])
    g = L.Shell(X, T, p)
    g.set_pressure_function("-1e-3*min(1, t/0.5)")
    g.apply_initial_conditions(u0, 0.0, -1e-3 * min(1, 2e-2 / 0.5))
    g.step(30, None)
    g2 = L.Shell(X, T, p)
    step, dt, _, _ = g2.load_state_file(os.path.join(d1, "shell_state0000000030.dat"))
    assert step == 30 and dt == g.dt()[0]
    for x, y in zip(g.get_state(), g2.get_state()):
        assert np.array_equal(x, y)
