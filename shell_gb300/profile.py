"""Steps of the benchmark workload with every kernel launched on its own, for
kernel profilers (the CUDA graphs of shl_step hold conditional nodes, whose
kernels profilers cannot replay one by one).

python -m shell_gb300.profile [--level 6] [--warmup 3] [--steps 5] [--squashed] [--contact linear|smooth|none]
    [--phases] [--variant V] [--start N] [--ensemble N]

--squashed starts from the double-layer state of the contact-mode benchmark
instead of the imperfect sphere; --start N first runs N steps of the ramp as
graph replays (not profiled kernels: give ncu a kernel filter), so that the
profiled steps lie later in the run; --phases also prints shl_profile_step's
per-phase event times (predictor, linked cells, elements, contact, gather,
volume) of one more step.  --ensemble N profiles the batched ensemble of the
benchmark instead (its first N shells: levels 3-5, FP32 element forces,
per-shell self-contact), at the start of its pressure ramp or, with
--squashed, with every shell flattened to a double layer.
"""
import argparse
import time

import numpy as np

from . import lib as L
from .workloads import RAMP_STEPS, ensemble_workload, pressure, squashed_state, workload


def run_ensemble(a):
    shells, params, scale, u0 = ensemble_workload(L, n_shells=a.ensemble)
    b = L.Batch(shells, params, pressure_scale=scale)
    if a.variant >= 0:
        b.set_element_variant(a.variant)
    n = a.warmup + a.steps
    if a.squashed:
        u = np.concatenate([squashed_state(X, seed=k) for k, (X, _) in enumerate(shells)])
        z = np.zeros_like(u)
        b.set_state(u, z, z)
        b.rebuild_contacts()
        table = np.zeros(n)
    else:
        b.apply_initial_conditions(u0, 0.0, -1.0 / RAMP_STEPS)
        table = -np.arange(1, n + 1, dtype=np.float64) / RAMP_STEPS
    b.step(a.warmup, table[:a.warmup], use_graph=False)
    t0 = time.perf_counter()
    r, st = b.step(a.steps, table[a.warmup:], use_graph=False)
    wall = time.perf_counter() - t0
    print("ensemble of %d shells, %d faces, %d steps in %.3f s (kernels launched one by one), status %d, pairs %d"
          % (b.n_shells, b.F, a.steps, wall, st, len(b.contact_state()["pairs"])))
    b.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--squashed", action="store_true")
    ap.add_argument("--contact", default="linear", choices=["linear", "smooth", "none"])
    ap.add_argument("--phases", action="store_true")
    ap.add_argument("--variant", type=int, default=-1, help="element-kernel variant (-1: the autotuned one)")
    ap.add_argument("--start", type=int, default=0, help="steps of the ramp run as graph replays first")
    ap.add_argument("--ensemble", type=int, default=0, help="profile the first N shells of the batched ensemble")
    a = ap.parse_args(argv)
    if a.ensemble:
        run_ensemble(a)
        return
    mode = {"linear": L.CONTACT_LINEAR, "smooth": L.CONTACT_SMOOTH, "none": L.CONTACT_NONE}[a.contact]
    X, T, p, u0 = workload(L, a.level, contact=mode)
    g = L.Shell(X, T, p)
    if a.variant >= 0:
        g.set_element_variant(a.variant)
    if a.squashed:
        u = squashed_state(X)
        z = np.zeros_like(u)
        g.set_state(u, z, z)
        g.rebuild_contacts()
        table = np.zeros(a.warmup + a.steps + 1)
    else:
        g.apply_initial_conditions(u0, 0.0, pressure(1))
        if a.start > 0:
            g.step(a.start, pressure(np.arange(1, a.start + 1)), use_graph=True)
        table = pressure(np.arange(a.start + 1, a.start + a.warmup + a.steps + 2))
    g.step(a.warmup, table[:a.warmup], use_graph=False)
    t0 = time.perf_counter()
    r, st = g.step(a.steps, table[a.warmup:a.warmup + a.steps], use_graph=False)
    wall = time.perf_counter() - t0
    print("faces %d, %d steps in %.3f s (kernels launched one by one), status %d, pairs %d, rebuilds %d"
          % (len(T), a.steps, wall, st, r.last.n_pairs, r.n_rebuilds))
    if a.phases:
        ms = g.profile_step(table[-1])
        print("  ".join("%s %.4f ms" % (n, m) for n, m in ms.items()))
    g.close()


if __name__ == "__main__":
    main()
