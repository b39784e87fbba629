"""Benchmark of the explicit shell time step on one GB300 (and N replicas).

Workload (the single-shell FP64 configuration): level-6 icosphere (40,962
nodes, 81,920 faces), orthotropic Koiter shell E1=1, E2=0.5, nu12=0.3,
G12=0.35, h/R=0.01, density 1, Rayleigh damping 0.05, dt=1e-4, external
pressure ramped from 0 to 2x the classical buckling pressure over 20,000
steps, seeded Gaussian normal imperfection of amplitude 1e-3 R, linear
self-contact with Coulomb friction mu=0.3 and linked cells of 2h.  Inputs are
synthetic (generated icosphere and seeded imperfection); there is no dataset.
Over its first 20,000 steps this shell does not buckle: it has no contact
pairs, and its candidate list is rebuilt about once every 20 steps.

A step is one Newmark step (ShellSystem::advance) of that shell; the metric is
face-steps per second.  The K timed steps are every S-th step of the run after
W warm-up steps, S = max(1, 1000 // K): they sample the first 1,000 steps at
an even stride, so candidate-list rebuilds enter at their rate.  Both arms
(the library and the CPU reference arm) time exactly these steps.
Reported:
  value      device throughput of the timed steps, each launched as one CUDA
             graph replay and bracketed by CUDA events on the library's
             stream, with L2 evicted (a 512 MB write) before each; the steps
             between them run untimed;
  e2e        the same steps through the C ABI with host buffers: per timed
             step the state (u, v, a) is copied in from pinned host memory,
             the step runs, and the state is copied back;
  run_value  the whole 10,000-step run, replayed back to back (16 steps per
             graph replay), one pair of CUDA events around it;
  parity     the 10,000-step run checked against the oracle every 100 steps
             (same-state force, step and candidate-list checks; the first
             1,000 steps also in lockstep), and the contact-heavy run;
  roofline   the element-force kernel timed live (events, cold L2) against
             its algorithmic bytes, the FP64-equivalent flops and the
             instruction issue rate;
  cpu_baseline  the CPU oracle on this host's cores on the same timed steps,
             with 3 threads (the reference launcher's setting) on a sample,
             and the full 20,000-step level-3 run;
  contact_modes  LINEAR and SMOOTH self-contact at a squashed, contact-heavy
             state of the same shell, with the CPU oracle on the same steps.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--level L]
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from shell_gb300.workloads import (ALPHA, AMPL, DT, G12, MU, NU12, RAMP_STEPS, RHO, SEED, ensemble_workload,  # noqa: E402
                                   classical_pressure, pressure, squashed_state, workload)

FLUSH_BYTES = 512 << 20
SAMPLE_SPAN = 1000   # the timed steps sample this many steps after the warm-up
RUN_STEPS = 10000    # the length of the level-6 FP64 run
# library kernels per step with self-contact: step start (k_begin_step, which also sets the
# condition of the step's rebuild IF node), element kernel, contact force, gather/corrector
# (which also predicts the next step), volume/measurement totals/end of step; plus, for each
# rebuild, the body of the IF node: two linked-cell passes of 27 kernels (10 pipeline +
# 3 x 3 scan + 8 contact CSR; the one not due returns at once) and the kernel between them
LAUNCHES_PER_STEP_CONTACT = 5
LAUNCHES_PER_REBUILD = 55
# algorithmic bytes of one face-step of the FP64 path: vertex state u, v, a read and written
# plus M^-1 and C (96 B per face), per-face constants (R, reference metric, forms, stiffness,
# JxW: 264 B), connectivity and CSR (96 B); intermediate force shares are not counted
STEP_BYTES_PER_FACE = 456
# FP64 flops of one regular face in the element kernel (count of the
# arithmetic in element_force<12>, fused multiply-add = 2)
ELEM_FLOPS_PER_FACE = 1372
# DRAM bytes (read + write) of one launch of the tuned element kernel (the
# one-round double-float shape, 544 threads per SM) on the level-6 shell, from
# one ncu --set full capture with caches flushed (46.3 MB read, 15.9 MB written)
ELEM_TRAFFIC_LEVEL6 = 62.2e6
# FP32 element path (the ensemble): about 300 algorithmic bytes per face-step with
# FP32 per-face constants; DRAM bytes of one launch on the 256-shell ensemble and its
# FP32-pipe utilisation, from one ncu --set full capture (673.4 MB read, 427.0 MB
# written: the force shares do not fit in L2 at this size)
ENS_BYTES_PER_FACE = 300
ENS_ELEM_TRAFFIC = 1100.4e6
ENS_ELEM_FP32_PIPE = 0.129
# warp instructions of one element-kernel launch on the level-6 shell (ncu
# smsp__inst_executed.sum of the same capture) and the issue peak: 4 schedulers
# per SM, one warp instruction per cycle each
ELEM_WARP_INST_LEVEL6 = 30.7e6
ISSUE_PER_SM_PER_CYCLE = 4


def stride_for(K):
    return max(1, SAMPLE_SPAN // K)


def line_config(level, F, V, K, W, world):
    """The `config` of both arms (identical, so the two lines compare)."""
    S = stride_for(K)
    return {"workload": "single shell, level-%d icosphere (%d faces, %d nodes), FP64 element forces and state, "
                        "self-contact + Coulomb friction (mu 0.3, linked cells 2h), pressure ramp to 2 p_cl over "
                        "%d steps (dt 1e-4)" % (level, F, V, RAMP_STEPS),
            "faces": F, "nodes": V,
            "timed_steps": "%d steps: every %d-th step of steps %d-%d, after %d warm-up steps" % (
                K, S, W + 1, W + S * K, W),
            "parallelism": "replicas (one shell per GPU; rank 0 times the CPU arm)" if world > 1 else "single",
            "l2": "GPU arm: evicted before every timed step (512 MB write); CPU arm: not applicable"}


def cpu_model():
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, text=True).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name") or ln.lower().startswith("vendor id"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def _timed_batch_steps(b, torch, K, flush):
    """K single-step graph replays of a batch, each bracketed by CUDA events on
    the batch's stream with L2 evicted before it; returns the summed ms."""
    stream = torch.cuda.ExternalStream(b.stream_handle())
    st = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    with torch.cuda.stream(stream):
        for k in range(K):
            flush.fill_(k)
            st[k].record(stream)
            b.step_enqueue(1)
            en[k].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(e) for a, e in zip(st, en))


def time_ensemble(L, torch, K, W, flush):
    """The 256-shell ensemble: K steps of its pressure ramp after W warm-up
    steps (no shell is in contact yet; every shell's linked-cell trigger runs),
    and K steps with every shell squashed to a double layer (zero pressure:
    each shell's candidate list is long and rebuilt as it moves)."""
    shells, params, scale, u0 = ensemble_workload(L)
    b = L.Batch(shells, params, pressure_scale=scale)
    ramp = lambda st: -np.asarray(st, dtype=np.float64) / RAMP_STEPS  # noqa: E731
    b.apply_initial_conditions(u0, 0.0, ramp(1))
    b.upload_pressure_table(ramp(np.arange(1, 1 + W + K)))
    b.step_enqueue(W)
    torch.cuda.synchronize()
    ms = _timed_batch_steps(b, torch, K, flush)
    rep, status = b.step_collect()
    _, nr0 = b.contact_stats()
    n_pairs = len(b.contact_state()["pairs"])
    # contact-heavy: every shell flattened to a double layer
    rng = np.random.default_rng(7)
    us = []
    for X, _ in shells:
        u = np.zeros_like(X)
        u[:, 2] = (0.0042 - 1.0) * X[:, 2]
        us.append((u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1))
    z = np.zeros(3 * b.V)
    b.set_state(np.concatenate(us), z, z)
    b.rebuild_contacts()
    b.upload_pressure_table(np.zeros(W + K))
    b.step_enqueue(W)
    torch.cuda.synchronize()
    _, nr1 = b.contact_stats()
    ms_c = _timed_batch_steps(b, torch, K, flush)
    rep_c, status_c = b.step_collect()
    _, nr2 = b.contact_stats()
    pairs_c = len(b.contact_state()["pairs"])
    F = b.F
    # the FP32 element kernel alone (CUDA events, L2 evicted before each launch)
    elem_ms = b.time_kernel(0, reps=10, flush_bytes=FLUSH_BYTES)
    elem_variant = b.element_variant()[1]
    b.close()
    hbm = 6800.0
    try:
        hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, ValueError, KeyError):
        pass
    ach = F * ENS_BYTES_PER_FACE / (elem_ms * 1e-3) / 1e9
    levels = [int(round(np.log(len(T) / 20) / np.log(4))) for _, T in shells]
    return {"value": F * K / (ms * 1e-3), "unit": "face-steps/s", "ms_per_step": ms / K, "shells": len(shells),
            "faces": int(F), "levels": {str(lv): levels.count(lv) for lv in (3, 4, 5)},
            "dtype": "f32 forces, f64 state and contact gaps", "contact": "linear + friction, per-shell linked cells",
            "steps": K, "status": int(status), "n_pairs": int(n_pairs), "shell_rebuilds_total": int(nr0.sum()),
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                         "traffic": ENS_ELEM_TRAFFIC, "kernel": "k_elements32", "variant": elem_variant,
                         "kernel_ms": elem_ms, "fp32_pipe_frac": ENS_ELEM_FP32_PIPE,
                         "algorithmic_bytes": "%d B per face-step x %d faces" % (ENS_BYTES_PER_FACE, F),
                         "note": "the FP32 element kernel of the batched path, timed live; traffic and FP32-pipe "
                                 "share from one ncu capture (the larger fraction, HBM, is the bound)"},
            "contact_heavy": {"value": F * K / (ms_c * 1e-3), "ms_per_step": ms_c / K, "n_pairs": int(pairs_c),
                              "shell_rebuilds_in_timed_steps": int((nr2 - nr1).sum()),
                              "status": int(status_c),
                              "state": "every shell squashed to a double layer, zero pressure"}}


def time_contact_modes(L, torch, K, W, flush, level, cpu=True):
    """Self-contact at a contact-heavy state: the level-`level` shell of the
    main workload squashed to a double layer (every face has candidates on the
    other layer), zero pressure, with the LINEAR (flat triangles) and SMOOTH
    (Loop limit surfaces) narrow phases: K timed steps each (L2 evicted before
    every step) after W warm-up steps, and the first candidate-list build.
    With `cpu`, the CPU oracle (all host threads) takes the same first build
    and the first steps from the same state (one step for SMOOTH, whose CPU
    step takes seconds)."""
    X, T, _, _ = workload(L, level)
    u = squashed_state(X)
    z = np.zeros_like(u)
    F = len(T)
    out = {"workload": "level-%d shell squashed to a double layer (gap 2 x 0.0042 |z|), zero pressure, steps "
                       "%d-%d" % (level, W + 1, W + K), "faces": F}
    for name, mode in (("linear", L.CONTACT_LINEAR), ("smooth", L.CONTACT_SMOOTH)):
        _, _, p, _ = workload(L, level, contact=mode)
        g = L.Shell(X, T, p)
        g.set_state(u, z, z)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.rebuild_contacts()
        build_s = time.perf_counter() - t0
        g.upload_pressure_table(np.zeros(W + K))
        g.step_enqueue(W)
        torch.cuda.synchronize()
        g.step_collect()
        stream = torch.cuda.ExternalStream(g.stream_handle())
        st = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.fill_(k)
                st[k].record(stream)
                g.step_enqueue(1)
                en[k].record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(e) for a, e in zip(st, en))
        rep, status = g.step_collect()
        out[name] = {"value": F * K / (ms * 1e-3), "unit": "face-steps/s", "ms_per_step": ms / K,
                     "n_pairs": int(rep.last.n_pairs), "Nc": int(rep.last.Nc), "n_rebuilds": int(rep.n_rebuilds),
                     "first_build_s": build_s, "status": int(status)}
        g.close()
        if cpu:
            import oracle as O

            lib = O.load()
            o = O.Oracle(X, T, p, threads=os.cpu_count())
            o.set_state(u, z, z)
            t0 = time.perf_counter()
            o.rebuild_contacts()
            cpu_build = time.perf_counter() - t0
            # one step with all host threads, one with 3 (the reference launcher's setting); the faster counts
            times = {}
            for k, t in enumerate(sorted({os.cpu_count(), min(3, os.cpu_count())}, reverse=True)):
                lib.oracle_set_threads(t)
                t0 = time.perf_counter()
                r, _ = o.step(1, np.zeros(1))
                times[t] = time.perf_counter() - t0
            o.close()
            best = min(times, key=times.get)
            out[name].update(cpu_value=F / times[best], cpu_ms_per_step=times[best] * 1e3,
                             cpu_first_build_s=cpu_build, cpu_threads=best,
                             cpu_steps="steps 1-%d from the squashed state, one step per thread count (%s), "
                                       "the faster counts" % (len(times), "/".join(str(t) for t in times)),
                             cpu_n_pairs=int(r.last.n_pairs))
    return out


def fp32_accuracy(L, steps=1000, level=7):
    """Level-7 shell, h/R = 0.005, E1/E2 = 4, pressure ramp to 3 p_cl over
    50,000 steps, self-contact on: FP32 element forces against FP64 (the FP64
    path equals the CPU oracle to 1e-12) -- per-vertex force error at the
    initial state and after `steps` steps, and the displacement drift."""
    import oracle as O

    h, e1, e2, s_end, ramp_steps = 0.005, 2.0, 0.5, 3.0, 50000
    X, T = L.icosphere(level)
    P = X[T]
    cell_mult = 2 * h / (P.max(axis=1) - P.min(axis=1)).max(axis=1).mean()
    E = np.sqrt(e1 * e2)
    nu = np.sqrt(NU12 * NU12 * e2 / e1)
    p_cl = 2 * E * h * h / np.sqrt(3 * (1 - nu * nu))
    common = dict(shell_mass_density=RHO, shell_young_modulus=e1, shell_young_modulus2=e2, shell_poisson_ratio=NU12,
                  shell_shear_modulus=G12 * E, thickness=h, damping_alpha=ALPHA, dt=DT,
                  shell_shell_contact=L.CONTACT_LINEAR, mu_s=MU, mu_d=MU, cell_size_mult=cell_mult)
    u0 = L.gaussian_normal_imperfection(X, AMPL, SEED).reshape(-1)
    table = -s_end * p_cl * np.arange(1, steps + 1) / ramp_steps
    out = {}
    runs = {}
    for name, prec in (("fp64", L.PREC_FP64), ("fp32", L.PREC_FP32)):
        g = L.Shell(X, T, L.default_params(precision=prec, **common))
        g.apply_initial_conditions(u0, 0.0, table[0])
        f0 = g.eval_forces(u0, np.zeros_like(u0), table[0])[0]
        r, st = g.step(steps, table)
        u, v, a = g.get_state()
        f1 = g.eval_forces(u, v, table[-1])[0]
        runs[name] = (f0, u, f1, st, r.steps_done)
        g.close()
    o = O.Oracle(X, T, L.default_params(**common), threads=os.cpu_count())
    f0_oracle = o.eval_forces(u0, np.zeros_like(u0), table[0])[0]
    o.close()

    def node_err(f, ref):
        d = np.linalg.norm((f - ref).reshape(-1, 3), axis=1)
        scale = np.linalg.norm(ref.reshape(-1, 3), axis=1).max()
        return {"max_node_rel": float(d.max() / scale), "l2_rel": float(np.linalg.norm(f - ref) / np.linalg.norm(ref))}

    f0_64, u_64, f1_64, st64, n64 = runs["fp64"]
    f0_32, u_32, f1_32, st32, n32 = runs["fp32"]
    out["workload"] = "level-%d shell (%d faces), h/R %.3f, E1/E2 4, ramp to 3 p_cl over %d steps, %d steps" % (
        level, len(T), h, ramp_steps, steps)
    out["force_error_initial_vs_oracle"] = node_err(f0_32, f0_oracle)
    out["fp64_vs_oracle_initial"] = node_err(f0_64, f0_oracle)
    out["force_error_after"] = node_err(f1_32, f1_64)
    out["displacement_drift"] = float(np.linalg.norm(u_32 - u_64) / np.linalg.norm(u_64 - u0))
    out["steps_done"] = [int(n64), int(n32)]
    return out


def cpu_sampled(X, T, p, u0, K, W, threads=None):
    """The CPU oracle on the timed steps of the benchmark: W warm-up steps,
    then K timed steps, every S-th step, the steps between untimed.  Without
    `threads`, the warm-up steps after the first try all host threads, half of
    them and 3 (the reference launcher's OMP_NUM_THREADS, script.pl:54), one
    step each, and the timed steps use the fastest: the oracle keeps the
    reference's critical-section assembly, which can scale worse than linearly."""
    import oracle as O

    lib = O.load()
    S = stride_for(K)
    n = os.cpu_count()
    cands = [threads] if threads else sorted({n, max(1, n // 2), min(3, n)}, reverse=True)
    o = O.Oracle(X, T, p, threads=cands[0])
    o.apply_initial_conditions(u0, 0.0, float(pressure(1)))
    o.step(1, pressure(np.array([1])))
    step, probe = 1, {}
    for t in cands:
        if step >= W:
            break
        lib.oracle_set_threads(t)
        t0 = time.perf_counter()
        o.step(1, pressure(np.array([step + 1])))
        probe[t] = time.perf_counter() - t0
        step += 1
    best = min(probe, key=probe.get) if probe else cands[0]
    lib.oracle_set_threads(best)
    if step < W:
        o.step(W - step, pressure(np.arange(step + 1, W + 1)))
        step = W
    secs, rebuilds, pairs = 0.0, 0, 0
    for _ in range(K):
        if S > 1:
            o.step(S - 1, pressure(np.arange(step + 1, step + S)))
            step += S - 1
        t0 = time.perf_counter()
        r, _ = o.step(1, pressure(np.array([step + 1])))
        secs += time.perf_counter() - t0
        step += 1
        rebuilds += r.n_rebuilds
        pairs = max(pairs, r.last.n_pairs)
    o.close()
    return {"value": len(T) * K / secs, "unit": "face-steps/s", "cores": best, "kind": "port",
            "sample": "the %d timed steps of the benchmark (every %d-th step of steps %d-%d), %.2f s timed, "
                      "OpenMP %d threads (fastest of %s on a warm-up step each)"
                      % (K, S, W + 1, W + S * K, secs, best, "/".join(str(t) for t in cands)),
            "thread_probe_s": {str(t): v for t, v in probe.items()},
            "n_rebuilds_timed": int(rebuilds), "n_pairs": int(pairs)}


def cpu_rate(X, T, p, u0, n_steps, threads, first_step=1, table=None):
    """CPU oracle face-steps/s over n_steps consecutive steps from the initial conditions."""
    import oracle as O

    o = O.Oracle(X, T, p, threads=threads)
    tbl = pressure(np.arange(first_step, first_step + n_steps)) if table is None else table
    o.apply_initial_conditions(u0, 0.0, float(tbl[0]))
    t0 = time.perf_counter()
    r, st = o.step(n_steps, tbl)
    secs = time.perf_counter() - t0
    o.close()
    return {"value": len(T) * n_steps / secs, "seconds": secs, "steps": int(r.steps_done), "threads": threads,
            "n_rebuilds": int(r.n_rebuilds), "status": int(st)}


def cpu_baseline_extras(api, level, threads_ref=3):
    """The CPU figures beside the main sample: the level-`level` workload at
    the reference launcher's 3 OpenMP threads (script.pl:54) on its first 100
    steps, and the whole 20,000-step level-3 run with all threads and with 3."""
    X, T, p, u0 = workload(api, level)
    out = {"cpu_model": cpu_model(), "host_threads": os.cpu_count(),
           "threads_%d" % threads_ref: dict(cpu_rate(X, T, p, u0, 100, threads_ref),
                                            sample="steps 1-100 of the level-%d workload" % level)}
    X3, T3, p3, u03 = workload(api, 3)
    out["level3_full_run"] = {
        "workload": "level-3 icosphere (1280 faces), same physics, all 20,000 steps of the ramp",
        "all_threads": cpu_rate(X3, T3, p3, u03, RAMP_STEPS, os.cpu_count()),
        "threads_%d" % threads_ref: cpu_rate(X3, T3, p3, u03, RAMP_STEPS, threads_ref)}
    return out


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, val in zip(names, f[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference's step (the
    reference itself does not build), all host threads, on the same timed
    steps of the same workload.  Inputs come from the oracle's own generators,
    so this process loads no part of the CUDA library."""
    if rank != 0:
        return
    import oracle as O
    from oracle import inputs as I

    O.build()
    W, K = args.warmup, args.steps
    X, T, p, u0 = workload(I, args.level)
    s = cpu_sampled(X, T, p, u0, K, W)
    line = {"metric": "shell face-steps/sec at 1 GB300", "value": s["value"], "unit": "face-steps/s",
            "n_gpus": world, "steps": K, "warmup": W, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": line_config(args.level, len(T), len(X), K, W, world),
            "cpu_baseline": {"value": s["value"], "unit": s["unit"], "cores": s["cores"], "kind": "port",
                             "sample": s["sample"], "cpu_model": cpu_model()},
            "e2e": {"value": s["value"], "unit": "face-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "status": {"n_rebuilds_timed": s["n_rebuilds_timed"], "n_pairs": s["n_pairs"]},
            "note": "the reference needs an unpublished libMesh fork and muparser and misses Contact.C; "
                    "its CPU step is timed through the oracle restatement"}
    print(json.dumps(line), flush=True)


def fresh_start(g, u0):
    """The run from its initial conditions again: empty candidate list, time 0."""
    g.set_contact_state(np.zeros((0, 2), dtype=np.uint32), du_sum=0.0)
    g.set_time(0.0, 0)
    g.apply_initial_conditions(u0, 0.0, float(pressure(1)))


def census(g, u0, K, W):
    """Candidate-list passes and pairs of every step of the sampled window
    (untimed; a collect after every step, which completes a deferred pass
    inside the step that asked for it)."""
    S = stride_for(K)
    n = W + S * K
    fresh_start(g, u0)
    g.upload_pressure_table(pressure(np.arange(1, n + 1)))
    rebuilds = np.zeros(n + 1, dtype=np.int64)
    pairs = np.zeros(n + 1, dtype=np.int64)
    for s in range(1, n + 1):
        g.step_enqueue(1)
        r, _ = g.step_collect()
        rebuilds[s], pairs[s] = r.n_rebuilds, r.last.n_pairs
    return rebuilds, pairs


def timed_sample(g, torch, u0, K, W, flush, dist=None, clock=None):
    """W warm-up steps, then K timed steps (every S-th step; the steps between
    run untimed), each one graph replay bracketed by CUDA events on the
    library's stream after an L2-evicting write.  Returns per-step ms."""
    S = stride_for(K)
    fresh_start(g, u0)
    g.upload_pressure_table(pressure(np.arange(1, W + S * K + 1)))
    g.step_enqueue(W)
    torch.cuda.synchronize()
    g.step_collect()
    stream = torch.cuda.ExternalStream(g.stream_handle())
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if clock:
        clock.__enter__()
    with torch.cuda.stream(stream):
        for k in range(K):
            if S > 1:
                g.step_enqueue(S - 1)
            flush.fill_(k)
            starts[k].record(stream)
            g.step_enqueue(1)
            ends[k].record(stream)
    torch.cuda.synchronize()
    if clock:
        clock.__exit__()
    if dist:
        dist.barrier()
    ms = [a.elapsed_time(e) for a, e in zip(starts, ends)]
    report, status = g.step_collect()
    return ms, report, status


def e2e_sample(g, torch, u0, K, W):
    """The timed steps through the C ABI with host buffers, called as a host
    program binds it (ctypes calls with the buffers' addresses): per timed
    step shl_set_state from pinned host memory, shl_step(1) and shl_get_state
    into pinned host memory; the steps between run untimed."""
    import ctypes

    from shell_gb300.lib import ShlError, ShlStepReport

    S = stride_for(K)
    fresh_start(g, u0)
    table = np.ascontiguousarray(pressure(np.arange(1, W + S * K + 1)), dtype=np.float64)
    g.step(W, table[:W])
    u, v, a = g.get_state()
    bufs = [torch.from_numpy(x).pin_memory() for x in (u, v, a)]
    hu, hv, ha = (b.numpy() for b in bufs)
    lib, h = g.lib, g.h
    pu, pv, pa = (ctypes.c_void_p(x.ctypes.data) for x in (hu, hv, ha))
    rep = ShlStepReport()
    rref = ctypes.byref(rep)
    step, secs = W, 0.0
    for _ in range(K):
        if S > 1:
            g.step(S - 1, table[step:step + S - 1])
            step += S - 1
            g.get_state(out=(hu, hv, ha))  # the host copy of the state before the timed step
        tp = ctypes.c_void_p(table.ctypes.data + 8 * step)
        t0 = time.perf_counter()
        s1 = lib.shl_set_state(h, pu, pv, pa)
        s2 = lib.shl_step(h, 1, tp, 1, rref)
        s3 = lib.shl_get_state(h, pu, pv, pa)
        secs += time.perf_counter() - t0
        for st, where in ((s1, "shl_set_state"), (s2, "shl_step"), (s3, "shl_get_state")):
            if st >= 100 or (st != 0 and where != "shl_step"):
                raise ShlError(st, where)
        step += 1
    return secs


def warmstart_leg(args):
    """Time to equilibrium (relative residual 1e-6, FP64) of held-out shells,
    relaxed from zero (plain) and from the learned prediction (warm), and
    the FP32 batched form (FP32 relaxation with FP64 defect correction, then
    an FP64 polish) against the plain FP64 form; the surrogate is trained on
    the GPU by the library's own kernels on equilibria the batched solver
    generates.  Pressures 0.15-0.5 p_cl: in the buckled range the collapsed
    shells do not reach the residual (profiles/warmstart_buckled_probe.md)."""
    from shell_gb300 import warmstart as WS
    t0 = time.perf_counter()
    lv = args.ws_level
    r = WS.experiment(n_train=args.ws_train, n_test=args.ws_test, seed=1, batch_size=512, train_iters=1500,
                      gen_tol=1e-5, gen_max=15000, tol=1e-6, max_steps=15000, level=lv, hidden=[512] * 4,
                      train_batch=128, s_range=(0.15, 0.5), contact=False, mixed=True,
                      log=lambda m: print(m, file=sys.stderr))
    t64 = r["test"]["fp64"]
    mix = r["test"]["fp32+fp64"]
    plain, warm = t64["plain"], t64["warm"]
    return {
        "workload": "level-%d shells (%d faces each), %d training / %d held-out problems; constant pressure "
                    "0.15-0.5 p_cl; explicit relaxation dt %g, mass damping %g; residual 1e-6 (FP64)"
                    % (lv, 20 * 4 ** lv, args.ws_train, args.ws_test, WS.DT, WS.DAMPING),
        "network": "8 -> 512 x 4 (GELU) -> %d, BF16 weights, FP32 accumulation, tcgen05 GEMMs" % (3 * (10 * 4 ** lv + 2)),
        "time_to_equilibrium": {
            "plain": {"median_steps": plain["median_steps"], "wall_s": plain["wall_s"],
                      "converged": plain["converged"]},
            "warm": {"median_steps": warm["median_steps"], "wall_s": warm["wall_s"], "converged": warm["converged"],
                     "fallbacks": warm["fallbacks"],
                     "equilibrium_within_1e-4_of_plain": warm["equilibrium_within_1e-4_of_plain"]},
            "steps_saved": (None if plain["median_steps"] is None or warm["median_steps"] is None
                            else 1.0 - warm["median_steps"] / plain["median_steps"])},
        "fp32_batched_vs_fp64": {
            "fp64_plain_face_steps_per_s": t64["plain"]["phases"][0]["face_steps_per_s"],
            "fp32_phase_face_steps_per_s": mix["plain"]["phases"][0]["face_steps_per_s"],
            "fp32_plus_fp64_wall_s": mix["plain"]["wall_s"], "fp64_wall_s": t64["plain"]["wall_s"],
            "fp32_plus_fp64_median_steps": mix["plain"]["median_steps"],
            "equilibrium_within_1e-4_of_fp64": mix.get("plain_vs_fp64_plain_within_1e-4")},
        "prediction_error_over_h": t64.get("prediction_error_over_h"),
        "training": r["training"], "generation": r["generation"],
        "seconds": time.perf_counter() - t0}


def run_value_leg(g, torch, u0, n_steps=RUN_STEPS):
    """The whole run back to back (graph replays of 16 steps), warm L2."""
    fresh_start(g, u0)
    g.upload_pressure_table(pressure(np.arange(1, n_steps + 1)))
    stream = torch.cuda.ExternalStream(g.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        g.step_enqueue(n_steps)
        e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    rep, st = g.step_collect()
    return {"value": g.F * n_steps / (ms * 1e-3), "unit": "face-steps/s", "ms_per_step": ms / n_steps,
            "steps": int(rep.steps_done), "n_rebuilds": int(rep.n_rebuilds), "n_pairs_last": int(rep.last.n_pairs),
            "status": int(st), "how": "steps 1-%d of the run, %d graph replays of 16 steps, one pair of CUDA events, "
                                      "warm L2" % (n_steps, (n_steps + 15) // 16)}


def parity_leg(L, level, n_steps, lockstep_steps, contact_steps):
    """The run checked against the oracle every 100 steps, and the
    contact-heavy run from the squashed state every 25 steps (oracle.protocol)."""
    import oracle as O
    from oracle import protocol

    X, T, p, u0 = workload(L, level)

    def summary(r):
        return {k: r[k] for k in ("steps", "checks", "check_every", "lockstep_steps", "same_state_bit_exact",
                                  "lockstep_equal", "worst", "n_rebuilds", "n_rebuilds_oracle_lockstep",
                                  "max_pairs", "max_Nc", "seconds")}

    out = {"tolerances": "forces and accelerations at the same state 1e-12 relative; one step from the same state "
                         "1e-12; pair lists, FP64 d^2 and stick flags bit for bit"}
    r = protocol.run(L, O, X, T, p, u0=u0, n_steps=n_steps, check_every=100, lockstep_steps=lockstep_steps,
                     pressure=pressure, threads=os.cpu_count())
    out["run"] = summary(r)
    if contact_steps > 0:
        u = squashed_state(X)
        z = np.zeros_like(u)
        rc = protocol.run(L, O, X, T, p, state0=(u, z, z), n_steps=contact_steps, check_every=25,
                          lockstep_steps=25, threads=os.cpu_count())
        out["contact"] = dict(summary(rc), workload="the same shell squashed to a double layer, zero pressure")
    return out


def run_ours(args, rank, world, dist):
    import torch

    import shell_gb300.lib as L

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    X, T, p, u0 = workload(L, args.level)
    F, V = len(T), len(X)
    W, K = args.warmup, args.steps
    S = stride_for(K)
    g = L.Shell(X, T, p)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    reb, pairs = census(g, u0, K, W)
    timed_idx = W + S * (np.arange(K) + 1)
    clk = ClockSampler(dev)
    ms_list, report, status = timed_sample(g, torch, u0, K, W, flush, dist, clk)
    ms = sum(ms_list)
    if dist:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = F * K * world / (ms * 1e-3)
    rebuild_steps = np.zeros(K, dtype=bool)
    rebuild_steps[:] = reb[timed_idx] > 0
    ms_arr = np.array(ms_list)
    window = {"n_rebuilds_timed": int(reb[timed_idx].sum()), "n_pairs_max": int(pairs[timed_idx].max()),
              "ms_plain_step_median": float(np.median(ms_arr[~rebuild_steps])) if (~rebuild_steps).any() else None,
              "ms_rebuild_step_median": float(np.median(ms_arr[rebuild_steps])) if rebuild_steps.any() else None,
              "n_rebuilds_window": int(reb[W + 1:].sum())}

    # the same timed steps with FP32 element forces (FP64 state and contact)
    fp32_value = None
    if args.fp32:
        p32 = L.default_params(**{k: getattr(p, k) for k, _ in L._PARAM_FIELDS if not k.startswith("pad")})
        p32.precision = L.PREC_FP32
        g32 = L.Shell(X, T, p32)
        ms32, _, _ = timed_sample(g32, torch, u0, K, W, flush)
        g32.close()
        fp32_value = F * K / (sum(ms32) * 1e-3)

    e2e_s = e2e_sample(g, torch, u0, K, W)
    e2e = F * K * world / e2e_s
    run_value = run_value_leg(g, torch, u0)

    ensemble = time_ensemble(L, torch, max(20, K // 4), W, flush) if args.ensemble else None
    contact_modes = (time_contact_modes(L, torch, 10, 2, flush, args.level, cpu=rank == 0)
                     if args.contact_modes else None)
    accuracy = fp32_accuracy(L) if args.accuracy else None
    warmstart = None
    if args.warmstart and rank == 0:
        warmstart = warmstart_leg(args)

    # roofline of the element kernel (live, cold L2), at the state after the run
    elem_ms = g.time_kernel(0, reps=20, flush_bytes=FLUSH_BYTES)
    elem_variant = g.element_variant()[1]
    fp64_peak = L.measure_fp64_peak()
    g.close()
    parity = (parity_leg(L, args.level, args.parity_steps, args.parity_lockstep, args.parity_contact)
              if args.parity_steps > 0 and rank == 0 else None)
    bytes_elem = F * STEP_BYTES_PER_FACE
    achieved_gbs = bytes_elem / (elem_ms * 1e-3) / 1e9
    achieved_tf = F * ELEM_FLOPS_PER_FACE / (elem_ms * 1e-3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s (of fallback)"
    clocks = clk.summary()
    sm_ghz = (clocks.get("sm_max_mhz") or 2070.0) / 1e3
    issue_peak = ISSUE_PER_SM_PER_CYCLE * 152 * sm_ghz  # G warp instructions / s
    if rank != 0:
        return
    cpu = None
    if args.cpu_baseline:
        cpu = cpu_sampled(X, T, p, u0, K, W)
        cpu["cpu_model"] = cpu_model()
        cpu.update(cpu_baseline_extras(L, args.level))
    line = {
        "metric": "shell face-steps/sec at 1 GB300", "value": value, "unit": "face-steps/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": line_config(args.level, F, V, K, W, world),
        "window": window,
        "run_value": run_value,
        "fp32_value": fp32_value,
        "ensemble": ensemble,
        "contact_modes": contact_modes,
        "fp32_accuracy": accuracy,
        "warmstart": warmstart,
        "parity": parity,
        "e2e": {"value": e2e, "unit": "face-steps/s", "h2d_bytes_per_step": 3 * 3 * V * 8,
                "d2h_bytes_per_step": 3 * 3 * V * 8,
                "how": "per timed step: shl_set_state from pinned host memory, shl_step(1), shl_get_state into "
                       "pinned host memory (the library reads and writes mapped page-locked buffers with one "
                       "kernel each way)"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": achieved_gbs / hbm,
                     "traffic": ELEM_TRAFFIC_LEVEL6 if args.level == 6 else None,
                     "traffic_note": "bytes per launch, ncu capture of the level-6 element kernel",
                     "algorithmic_bytes": "%d B per face-step x %d faces" % (STEP_BYTES_PER_FACE, F),
                     "kernel": "k_elements", "variant": elem_variant,
                     "kernel_ms": elem_ms, "peak_source": hbm_src,
                     "issue": {"warp_inst_per_launch": ELEM_WARP_INST_LEVEL6 if args.level == 6 else None,
                               "achieved_ginst_s": (ELEM_WARP_INST_LEVEL6 / (elem_ms * 1e-3) / 1e9
                                                    if args.level == 6 else None),
                               "peak_ginst_s": issue_peak,
                               "frac": (ELEM_WARP_INST_LEVEL6 / (elem_ms * 1e-3) / 1e9 / issue_peak
                                        if args.level == 6 else None),
                               "note": "instruction issue: the bound of the double-float element kernel "
                                       "(4 warp instructions per SM per cycle at the sampled max SM clock)"},
                     "fp64": {"achieved_tflops": achieved_tf, "peak_tflops": fp64_peak,
                              "frac": achieved_tf / fp64_peak,
                              "flops": "FP64-equivalent flops of the element arithmetic (executed as float "
                                       "pairs on the FP32 pipe by the double-float variants)",
                              "peak_source": "DFMA register loop measured in this run"}},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": LAUNCHES_PER_STEP_CONTACT * S * K + LAUNCHES_PER_REBUILD * int(reb[W + 1:].sum()),
        "status": {"worst_problem": report.worst_problem, "steps_done": report.steps_done,
                   "n_rebuilds": report.n_rebuilds, "n_pairs": report.last.n_pairs},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--cpu-baseline", type=int, default=1, help="time the CPU oracle beside the GPU (rank 0)")
    ap.add_argument("--fp32", type=int, default=1, help="also time the FP32 element-force mode")
    ap.add_argument("--ensemble", type=int, default=1, help="also time the 256-shell batched ensemble")
    ap.add_argument("--accuracy", type=int, default=1, help="also report the level-7 FP32-vs-FP64 accuracy")
    ap.add_argument("--contact-modes", type=int, default=1,
                    help="also time LINEAR and SMOOTH self-contact at a squashed (contact-heavy) state")
    ap.add_argument("--parity-steps", type=int, default=RUN_STEPS,
                    help="steps of the run checked against the oracle every 100 steps (0 = no parity leg)")
    ap.add_argument("--parity-lockstep", type=int, default=1000, help="of these, steps also run by the oracle")
    ap.add_argument("--parity-contact", type=int, default=100, help="steps of the contact-heavy parity run")
    ap.add_argument("--warmstart", type=int, default=1,
                    help="also run the learned warm-start study: time to equilibrium, warm against plain start "
                         "and FP32 batched against FP64 plain (level-4 shells by default)")
    ap.add_argument("--ws-level", type=int, default=4)
    ap.add_argument("--ws-train", type=int, default=448)
    ap.add_argument("--ws-test", type=int, default=64)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "ours":
        import __graft_entry__

        __graft_entry__.build()
    if world > 1:
        import torch
        import torch.distributed as tdist

        if args.impl == "ours":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl" if args.impl == "ours" else "gloo")
        dist = tdist
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, dist)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
