"""Parity protocol of the level-6 FP64 workload (CUDA library against the oracle).

TEST INFRASTRUCTURE ONLY: the oracle is the checker.  Used by
tests/test_gpu_level6_protocol.py and by the parity leg of bench.py.

A run of the library is checked every `check_every` steps in two ways:

  lockstep   the oracle runs the same steps from the same initial conditions
             (for the first `lockstep_steps` steps): the states (u, v, a),
             the rebuild schedule of the candidate list (count per interval)
             and the candidate pairs are compared at every check.  Before
             buckling the two trajectories stay within roundoff of each other;
             with friction a 1e-14 difference can flip a stick/slip decision,
             after which the trajectories legitimately part;
  same state at every check the library's full state (u, v, a, time, step,
             candidate list with stick flags, spring origins, d^2 and du_sum)
             is loaded into a fresh library context and a fresh oracle.  Both
             rebuild the candidate list at that state (the forced rebuild of
             apply_initial_conditions after a load, ShellSystem.C:855-888):
             the sorted pair lists must be equal bit for bit (pairs, d^2 bits,
             stick flags).  Both then evaluate the forces at the Newmark
             prediction of the next step (ShellSystem.C:972-1008): f and a
             within `force_tol` relative; the contact state after the
             evaluation must again agree bit for bit (friction updates).
             Both are then reloaded and take one step: u, v, a within 1e-12
             relative and the pair lists bit for bit.

The schedule being replicated is ShellSystem::advance (ShellSystem.C:952-1122)
with its candidate-list rebuilds (ShellSystem.C:1910-2135, trigger at 1919 and
2016-2027).
"""
import time

import numpy as np


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


def _same_contacts(cg, co):
    """Pairs, d^2 bits and stick flags equal; spring origins within 1e-12 (the
    contact stiffness uses element areas of the library's element kernel)."""
    return (cg["pairs"].shape == co["pairs"].shape and np.array_equal(cg["pairs"], co["pairs"])
            and np.array_equal(_bits(cg["d2"]), _bits(co["d2"])) and np.array_equal(cg["stick"], co["stick"])
            and rel(cg["origin"], co["origin"]) <= 1e-12)


def _load(ctx, state):
    u, v, a, t, step, c = state
    ctx.set_state(u, v, a)
    ctx.set_time(t, step)
    ctx.set_contact_state(c["pairs"], c["stick"], c["origin"], c["d2"], c["du_sum"])


def same_state_check(g2, o2, state, pressure_next, params):
    """One same-state check (see the module text); returns its errors."""
    u, v, a = state[0], state[1], state[2]
    dt, beta, gamma = params.dt, params.newmark_beta, params.newmark_gamma
    out = {}
    for ctx in (g2, o2):
        _load(ctx, state)
        ctx.rebuild_contacts()
    cg, co = g2.contact_state(), o2.contact_state()
    out["pairs_rebuild_equal"] = _same_contacts(cg, co)
    out["n_pairs"] = int(len(co["pairs"]))
    # forces at the prediction of the next step (ShellSystem.C:972-989)
    up = u + dt * v + dt * dt * (0.5 - beta) * a
    vp = v + (1.0 - gamma) * dt * a
    fg, ag, eg, sg = g2.eval_forces(up, vp, pressure_next)
    fo, ao, eo, so = o2.eval_forces(up, vp, pressure_next)
    out["force_rel"] = rel(fg, fo)
    out["accel_rel"] = rel(ag, ao)
    out["Nc"] = int(eo["Nc"])
    out["status_equal"] = sg == so
    out["pairs_eval_equal"] = _same_contacts(g2.contact_state(), o2.contact_state())
    # one step from the same state
    for ctx in (g2, o2):
        _load(ctx, state)
        ctx.rebuild_contacts()
    rg, sg = g2.step(1, np.array([pressure_next]))
    ro, so = o2.step(1, np.array([pressure_next]))
    sg_, so_ = g2.get_state(), o2.get_state()
    out["step_u_rel"] = rel(sg_[0] - u, so_[0] - u)  # the step's increment
    out["step_v_rel"] = rel(sg_[1], so_[1])
    out["step_a_rel"] = rel(sg_[2], so_[2])
    out["pairs_step_equal"] = _same_contacts(g2.contact_state(), o2.contact_state()) and sg == so
    return out


def run(L, O, X, T, params, u0=None, state0=None, n_steps=1000, check_every=100, lockstep_steps=None,
        pressure=None, threads=None, log=None):
    """Run the library for n_steps from u0 (apply_initial_conditions) or from
    state0 = (u, v, a) (set_state + a forced candidate-list build), checking it
    every check_every steps; returns a summary with the worst errors.
    pressure(steps) gives the pressure of 1-based steps."""
    lockstep_steps = n_steps if lockstep_steps is None else lockstep_steps
    pressure = pressure or (lambda s: np.zeros(np.size(s)))
    t_start = time.perf_counter()
    g = L.Shell(X, T, params)
    g2 = L.Shell(X, T, params)
    o = O.Oracle(X, T, params, threads=threads) if lockstep_steps > 0 else None
    o2 = O.Oracle(X, T, params, threads=threads)
    p1 = float(np.atleast_1d(pressure(1))[0])
    if state0 is None:
        g.apply_initial_conditions(u0, 0.0, p1)
        if o:
            o.apply_initial_conditions(u0, 0.0, p1)
    else:
        for ctx in [g] + ([o] if o else []):
            ctx.set_state(*state0)
            ctx.rebuild_contacts()
    checks = []
    worst = {"force_rel": 0.0, "accel_rel": 0.0, "step_u_rel": 0.0, "step_v_rel": 0.0, "step_a_rel": 0.0,
             "lockstep_u_rel": 0.0, "lockstep_v_rel": 0.0, "lockstep_a_rel": 0.0}
    same_state_exact = lockstep_equal = True
    rebuilds_g = rebuilds_o = 0
    max_pairs = max_nc = 0
    step = 0
    while step < n_steps:
        n = min(check_every, n_steps - step)
        table = np.atleast_1d(pressure(np.arange(step + 1, step + n + 1)))
        rg, sg = g.step(n, table)
        rebuilds_g += rg.n_rebuilds
        rec = {"step": step + n, "status": int(sg), "n_rebuilds": int(rg.n_rebuilds)}
        if o is not None and step + n <= lockstep_steps:
            ro, so = o.step(n, table)
            rebuilds_o += ro.n_rebuilds
            ug, vg, ag = g.get_state()
            uo, vo, ao = o.get_state()
            rec.update(lockstep_u_rel=rel(ug, uo), lockstep_v_rel=rel(vg, vo), lockstep_a_rel=rel(ag, ao),
                       lockstep_rebuilds_equal=rg.n_rebuilds == ro.n_rebuilds and sg == so)
            cg, co = g.contact_state(), o.contact_state()
            rec["lockstep_pairs_equal"] = bool(np.array_equal(cg["pairs"], co["pairs"]))
            lockstep_equal &= rec["lockstep_rebuilds_equal"] and rec["lockstep_pairs_equal"]
            for k in ("lockstep_u_rel", "lockstep_v_rel", "lockstep_a_rel"):
                worst[k] = max(worst[k], rec[k])
        u, v, a = g.get_state()
        t, st = g.get_time()
        c = g.contact_state()
        chk = same_state_check(g2, o2, (u, v, a, t, st, c), float(np.atleast_1d(pressure(step + n + 1))[0]),
                               params)
        rec.update(chk)
        same_state_exact &= chk["pairs_rebuild_equal"] and chk["pairs_eval_equal"] and chk["pairs_step_equal"] and \
            chk["status_equal"]
        for k in ("force_rel", "accel_rel", "step_u_rel", "step_v_rel", "step_a_rel"):
            worst[k] = max(worst[k], chk[k])
        max_pairs = max(max_pairs, chk["n_pairs"])
        max_nc = max(max_nc, chk["Nc"])
        checks.append(rec)
        if log:
            log("step %d: pairs %d Nc %d rebuilds %d force %.2e step-u %.2e %s" % (
                rec["step"], chk["n_pairs"], chk["Nc"], rg.n_rebuilds, chk["force_rel"], chk["step_u_rel"],
                "ok" if same_state_exact else "MISMATCH"))
        step += n
        if sg >= 3:
            break
    for ctx in (g, g2, o, o2):
        if ctx is not None:
            ctx.close()
    return {"steps": step, "checks": len(checks), "check_every": check_every, "lockstep_steps": min(lockstep_steps, step),
            "same_state_bit_exact": bool(same_state_exact), "lockstep_equal": bool(lockstep_equal), "worst": worst, "n_rebuilds": int(rebuilds_g),
            "n_rebuilds_oracle_lockstep": int(rebuilds_o), "max_pairs": int(max_pairs), "max_Nc": int(max_nc),
            "seconds": time.perf_counter() - t_start, "records": checks}
