"""The level-6 FP64 workload checked against the oracle every 100 steps.

Workload: the level-6 icosphere shell (81,920 faces) of the benchmark, FP64,
self-contact with friction on, pressure ramped to 2 p_cl over 20,000 steps.
Before buckling it has no contact pairs, but its candidate list is rebuilt
about every 20 steps.  A second run starts the same shell from a state
squashed to a double layer (1.6 M candidate pairs, contact and friction in
every step) to check the contact pipeline through rebuilds.

Tolerances: forces and accelerations at the same state within 1e-12 relative;
one step from the same state within 1e-12 (u increment, v, a); candidate pair
lists after a rebuild, after a force evaluation and after a step equal bit for
bit (pairs, FP64 d^2 bits, stick flags).  Lockstep trajectories (the oracle
running the same steps) before buckling: the same rebuild schedule and pair
lists, states within 1e-9.
"""
import os

import numpy as np
import pytest

import oracle as O
from oracle import protocol
from shell_gb300 import lib as L
from shell_gb300.workloads import pressure, squashed_state, workload

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
STEP_TOL = 1e-12
TRAJ_TOL = 1e-9


def test_level6_workload_every_100_steps(cuda_ok):
    X, T, p, u0 = workload(L, 6)
    r = protocol.run(L, O, X, T, p, u0=u0, n_steps=1000, check_every=100, pressure=pressure,
                     threads=os.cpu_count())
    w = r["worst"]
    assert r["steps"] == 1000 and r["checks"] == 10
    assert r["n_rebuilds"] > 10, "the run must rebuild its candidate list"
    assert r["same_state_bit_exact"], [c for c in r["records"] if not c["pairs_step_equal"]]
    assert r["lockstep_equal"], "same rebuild schedule and pair lists as the oracle"
    assert r["n_rebuilds"] == r["n_rebuilds_oracle_lockstep"]
    assert w["force_rel"] < FORCE_TOL and w["accel_rel"] < FORCE_TOL, w
    assert max(w["step_u_rel"], w["step_v_rel"], w["step_a_rel"]) < STEP_TOL, w
    assert max(w["lockstep_u_rel"], w["lockstep_v_rel"], w["lockstep_a_rel"]) < TRAJ_TOL, w


def test_level6_contact_every_25_steps(cuda_ok):
    X, T, p, _ = workload(L, 6)
    u = squashed_state(X)
    z = np.zeros_like(u)
    r = protocol.run(L, O, X, T, p, state0=(u, z, z), n_steps=100, check_every=25, lockstep_steps=25,
                     threads=os.cpu_count())
    w = r["worst"]
    assert r["max_pairs"] > 100000 and r["max_Nc"] > 10000, "the squashed state is in contact"
    assert r["n_rebuilds"] > 0
    assert r["same_state_bit_exact"]
    assert w["force_rel"] < FORCE_TOL and w["accel_rel"] < FORCE_TOL, w
    assert max(w["step_u_rel"], w["step_v_rel"], w["step_a_rel"]) < STEP_TOL, w
