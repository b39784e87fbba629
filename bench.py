"""Benchmark of the explicit shell time step on one GB300 (and N replicas).

Workload (the single-shell FP64 configuration): level-6 icosphere (40,962
nodes, 81,920 faces), orthotropic Koiter shell E1=1, E2=0.5, nu12=0.3,
G12=0.35, h/R=0.01, density 1, Rayleigh damping 0.05, dt=1e-4, external
pressure ramped from 0 to 2x the classical buckling pressure over 20,000
steps, seeded Gaussian normal imperfection of amplitude 1e-3 R, linear
self-contact with Coulomb friction mu=0.3 and linked cells of 2h.  Inputs are
synthetic (generated icosphere and seeded imperfection); there is no dataset.

A step is one Newmark step (ShellSystem::advance) of that shell; the metric is
face-steps per second.  Reported:
  value      device throughput of the timed steps, each step launched as one
             CUDA graph and bracketed by CUDA events on the library's stream,
             with L2 evicted (a 512 MB write) before every step;
  e2e        the same steps through the C ABI with host buffers: per step the
             state (u, v, a) is copied from pinned host memory, one step runs,
             and the state is copied back;
  roofline   the element-force kernel timed live (events, cold L2) against
             its algorithmic bytes and FP64 flops;
  cpu_baseline  the CPU oracle on this host's cores on a bounded sample;
  contact_modes  LINEAR and SMOOTH self-contact at a squashed, contact-heavy
             state of the same shell (10 steps each).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--level L]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from shell_gb300.workloads import (ALPHA, AMPL, DT, G12, MU, NU12, RAMP_STEPS, RHO, SEED,  # noqa: E402
                                   classical_pressure, pressure, squashed_state, workload)

FLUSH_BYTES = 512 << 20
# library kernels per step with self-contact: step start (k_begin_step, which also sets the
# condition of the step's rebuild IF node), element kernel, contact force, gather/corrector
# (which also predicts the next step), volume/measurement totals/end of step; plus, for each
# rebuild, the body of the IF node: two linked-cell passes of 27 kernels (10 pipeline +
# 3 x 3 scan + 8 contact CSR; the one not due returns at once) and the kernel between them
LAUNCHES_PER_STEP_CONTACT = 5
LAUNCHES_PER_REBUILD = 55
# element kernel (double-float FP64 path): per-face constants as float pairs
# (38 fields x 8 B), patch ids, force shares (float pairs), element fields,
# face permutation (bytes); per-node predicted displacement (bytes)
ELEM_BYTES_PER_FACE = 38 * 8 + 12 * 4 + 36 * 8 + 5 * 8 + 4
ELEM_BYTES_PER_NODE = 24
# FP64 flops of one regular face in the element kernel (count of the
# arithmetic in element_force<12>, fused multiply-add = 2)
ELEM_FLOPS_PER_FACE = 1372
# DRAM bytes (read + write) of one element-kernel launch on the level-6 shell,
# from one ncu --set full capture with caches flushed (38.6 MB read, 3.4 MB
# written; the force shares stay in the 129 MB L2 for the gather)
ELEM_TRAFFIC_LEVEL6 = 42.0e6


def ensemble_workload(L, n_shells=256, seed=0):
    """256 shells, levels uniform over 3/4/5, per-shell parameters from a seed:
    E1/E2 log-uniform in [0.2, 5] (E1 E2 = 1), h/R log-uniform in [0.005, 0.05],
    pressure ramp end uniform in [1.2, 3] p_cl of the shell, imperfection
    amplitude log-uniform in [1e-4, 1e-2] R; FP32 element forces."""
    rng = np.random.default_rng(seed)
    meshes = {lv: L.icosphere(lv) for lv in (3, 4, 5)}
    shells, params, scale, u0 = [], [], [], []
    for k in range(n_shells):
        lv = int(rng.integers(3, 6))
        r = float(np.exp(rng.uniform(np.log(0.2), np.log(5.0))))
        h = float(np.exp(rng.uniform(np.log(0.005), np.log(0.05))))
        s = float(rng.uniform(1.2, 3.0))
        amp = float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-2))))
        e1, e2 = np.sqrt(r), 1.0 / np.sqrt(r)
        E = np.sqrt(e1 * e2)
        nu = np.sqrt(NU12 * NU12 * e2 / e1)
        p_cl = 2 * E * h * h / np.sqrt(3 * (1 - nu * nu))
        X, T = meshes[lv]
        params.append(L.default_params(shell_mass_density=RHO, shell_young_modulus=e1, shell_young_modulus2=e2,
                                       shell_poisson_ratio=NU12, shell_shear_modulus=G12 * E, thickness=h,
                                       damping_alpha=ALPHA, dt=DT, shell_shell_contact=L.CONTACT_NONE,
                                       precision=L.PREC_FP32))
        shells.append((X, T))
        scale.append(s * p_cl)
        u0.append(L.gaussian_normal_imperfection(X, amp, seed * 100000 + k).reshape(-1))
    return shells, params, np.array(scale), np.concatenate(u0)


def time_ensemble(L, torch, K, W, flush):
    shells, params, scale, u0 = ensemble_workload(L)
    b = L.Batch(shells, params, pressure_scale=scale)
    ramp = lambda st: -np.asarray(st, dtype=np.float64) / RAMP_STEPS  # noqa: E731
    b.apply_initial_conditions(u0, 0.0, ramp(1))
    b.upload_pressure_table(ramp(np.arange(1, 1 + W + K)))
    b.step_enqueue(W)
    torch.cuda.synchronize()
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
    ms = sum(a.elapsed_time(e) for a, e in zip(st, en))
    rep, status = b.step_collect()
    F = b.F
    b.close()
    levels = [int(round(np.log(len(T) / 20) / np.log(4))) for _, T in shells]
    return {"value": F * K / (ms * 1e-3), "unit": "face-steps/s", "ms_per_step": ms / K, "shells": len(shells),
            "faces": int(F), "levels": {str(lv): levels.count(lv) for lv in (3, 4, 5)}, "dtype": "f32 forces, f64 state",
            "steps": K, "status": int(status)}


def time_contact_modes(L, torch, K, W, flush, level):
    """Self-contact at a contact-heavy state: the level-`level` shell of the
    main workload squashed to a double layer (every face has candidates on the
    other layer), zero pressure, with the LINEAR (flat triangles) and SMOOTH
    (Loop limit surfaces) narrow phases: K timed steps each (L2 evicted before
    every step) after W warm-up steps, and the first candidate-list build."""
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


def cpu_sample(X, T, p, u0, seconds=10.0, threads=None):
    """CPU oracle on the same workload: steps until about `seconds` elapsed."""
    import oracle as O

    threads = threads or os.cpu_count()
    o = O.Oracle(X, T, p, threads=threads)
    o.apply_initial_conditions(u0, 0.0, pressure(1))
    o.step(1, pressure([1]))
    t0 = time.perf_counter()
    o.step(2, pressure([2, 3]))
    per = (time.perf_counter() - t0) / 2
    n = int(max(2, min(2000, seconds / max(per, 1e-6))))
    t0 = time.perf_counter()
    o.step(n, pressure(np.arange(4, 4 + n)))
    dt = time.perf_counter() - t0
    o.close()
    return {"value": len(T) * n / dt, "unit": "face-steps/s", "cores": threads, "kind": "port",
            "sample": "%d steps (steps 4-%d) of the level-%d workload, %.1f s, OpenMP %d threads"
                      % (n, 3 + n, int(round(np.log(len(T) / 20) / np.log(4))), dt, threads)}


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
    reference itself does not build), all host threads, same workload."""
    import shell_gb300.lib as L

    if rank != 0:
        return
    X, T, p, u0 = workload(L, args.level)
    s = cpu_sample(X, T, p, u0, seconds=args.cpu_seconds)
    line = {"metric": "shell face-steps/sec at 1 GB300", "value": s["value"], "unit": "face-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "single shell, level-%d icosphere (%d faces), FP64, self-contact + friction"
                                   % (args.level, len(T)), "faces": int(len(T)), "nodes": int(len(X)),
                       "parallelism": "replicas", "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": s["value"], "unit": s["unit"], "cores": s["cores"], "kind": "port",
                             "sample": s["sample"]},
            "e2e": {"value": s["value"], "unit": "face-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference needs an unpublished libMesh fork and muparser and misses Contact.C; "
                    "its CPU step is timed through the oracle restatement"}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import torch

    import shell_gb300.lib as L

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    X, T, p, u0 = workload(L, args.level)
    F, V = len(T), len(X)
    g = L.Shell(X, T, p)
    g.apply_initial_conditions(u0, 0.0, pressure(1))
    stream = torch.cuda.ExternalStream(g.stream_handle())
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    W, K = args.warmup, args.steps
    g.upload_pressure_table(pressure(np.arange(1, 1 + W + K)))
    # warm-up (graph instantiation, first rebuilds); the report then covers the timed steps only
    g.step_enqueue(W)
    torch.cuda.synchronize()
    g.step_collect()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.fill_(k)
                starts[k].record(stream)
                g.step_enqueue(1)
                ends[k].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    report, status = g.step_collect()
    if dist:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = F * K * world / (ms * 1e-3)

    # the same workload with FP32 element forces (FP64 state and contact), cold L2 per step
    fp32_value = None
    if args.fp32:
        p32 = L.default_params(**{k: getattr(p, k) for k, _ in L._PARAM_FIELDS if not k.startswith("pad")})
        p32.precision = L.PREC_FP32
        g32 = L.Shell(X, T, p32)
        g32.apply_initial_conditions(u0, 0.0, pressure(1))
        s32 = torch.cuda.ExternalStream(g32.stream_handle())
        g32.upload_pressure_table(pressure(np.arange(1, 1 + W + K)))
        g32.step_enqueue(W)
        torch.cuda.synchronize()
        st32 = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        en32 = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        with torch.cuda.stream(s32):
            for k in range(K):
                flush.fill_(k)
                st32[k].record(s32)
                g32.step_enqueue(1)
                en32[k].record(s32)
        torch.cuda.synchronize()
        ms32 = sum(a.elapsed_time(b) for a, b in zip(st32, en32))
        g32.step_collect()
        g32.close()
        fp32_value = F * K / (ms32 * 1e-3)

    ensemble = time_ensemble(L, torch, max(20, K // 4), W, flush) if args.ensemble else None
    contact_modes = time_contact_modes(L, torch, 10, 2, flush, args.level) if args.contact_modes else None
    accuracy = fp32_accuracy(L) if args.accuracy else None
    warmstart = None
    if args.warmstart:
        from shell_gb300 import warmstart as WS
        warmstart = WS.experiment(n_train=args.ws_train, n_test=args.ws_test, log=lambda m: print(m, file=sys.stderr))

    # warm continuous throughput (informative): K steps back to back, one graph replay per 16 steps
    g.upload_pressure_table(pressure(np.arange(1 + W + K, 1 + W + 2 * K)))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        g.step_enqueue(K)
        e1.record(stream)
    torch.cuda.synchronize()
    warm = F * K / (e0.elapsed_time(e1) * 1e-3)
    g.step_collect()

    # e2e through the C ABI with pinned host buffers
    u, v, a = g.get_state()
    hu = torch.from_numpy(u).pin_memory()
    hv = torch.from_numpy(v).pin_memory()
    ha = torch.from_numpy(a).pin_memory()
    nu_, nv_, na_ = hu.numpy(), hv.numpy(), ha.numpy()
    Ke = max(8, K // 4)
    pt = pressure(np.arange(1 + W + 2 * K, 1 + W + 2 * K + Ke))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(Ke):
        g.set_state(nu_, nv_, na_)
        g.step(1, pt[k:k + 1])
        g.get_state(out=(nu_, nv_, na_))
    e2e_s = time.perf_counter() - t0
    e2e = F * Ke * world / e2e_s

    # roofline of the element kernel (live, cold L2)
    elem_ms = g.time_kernel(0, reps=20, flush_bytes=FLUSH_BYTES)
    elem_variant = g.element_variant()[1]
    fp64_peak = L.measure_fp64_peak()
    g.close()
    bytes_elem = F * ELEM_BYTES_PER_FACE + V * ELEM_BYTES_PER_NODE
    achieved_gbs = bytes_elem / (elem_ms * 1e-3) / 1e9
    achieved_tf = F * ELEM_FLOPS_PER_FACE / (elem_ms * 1e-3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    if rank != 0:
        return
    cpu = cpu_sample(X, T, p, u0, seconds=args.cpu_seconds) if args.cpu_seconds > 0 else None
    line = {
        "metric": "shell face-steps/sec at 1 GB300", "value": value, "unit": "face-steps/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "single shell, level-%d icosphere (%d faces, %d nodes), FP64 element forces and "
                               "state, self-contact + Coulomb friction, pressure ramp to 2 p_cl over %d steps, "
                               "steps %d-%d of the run" % (args.level, F, V, RAMP_STEPS, W + 1, W + K),
                   "faces": F, "nodes": V, "parallelism": "replicas (one shell per GPU)" if world > 1 else "single",
                   "l2": "evicted before every timed step (512 MB write)"},
        "warm_value": warm,
        "fp32_value": fp32_value,
        "ensemble": ensemble,
        "contact_modes": contact_modes,
        "fp32_accuracy": accuracy,
        "warmstart": warmstart,
        "e2e": {"value": e2e, "unit": "face-steps/s", "h2d_bytes_per_step": 3 * 3 * V * 8,
                "d2h_bytes_per_step": 3 * 3 * V * 8,
                "how": "per step: shl_set_state from pinned host memory, shl_step(1), shl_get_state into pinned host memory (the library reads and writes mapped page-locked buffers with one kernel each way)"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": achieved_gbs / hbm,
                     "traffic": ELEM_TRAFFIC_LEVEL6 if args.level == 6 else None,
                     "traffic_note": "bytes per launch, ncu capture of the level-6 element kernel",
                     "kernel": "k_elements", "variant": elem_variant,
                     "kernel_ms": elem_ms, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                     "fp64": {"achieved_tflops": achieved_tf, "peak_tflops": fp64_peak,
                              "frac": achieved_tf / fp64_peak,
                              "flops": "FP64-equivalent flops of the element arithmetic (executed as float "
                                       "pairs on the FP32 pipe by the double-float variants)",
                              "peak_source": "DFMA register loop measured in this run"}},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": LAUNCHES_PER_STEP_CONTACT * K + LAUNCHES_PER_REBUILD * report.n_rebuilds,
        "status": {"worst_problem": report.worst_problem, "steps_done": report.steps_done,
                   "n_rebuilds": report.n_rebuilds, "n_pairs": report.last.n_pairs},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--fp32", type=int, default=1, help="also time the FP32 element-force mode")
    ap.add_argument("--ensemble", type=int, default=1, help="also time the 256-shell batched ensemble")
    ap.add_argument("--accuracy", type=int, default=1, help="also report the level-7 FP32-vs-FP64 accuracy")
    ap.add_argument("--contact-modes", type=int, default=1,
                    help="also time LINEAR and SMOOTH self-contact at a squashed (contact-heavy) state")
    ap.add_argument("--warmstart", type=int, default=0,
                    help="also run the learned warm-start study (level-5 shells; minutes of GPU time)")
    ap.add_argument("--ws-train", type=int, default=3584)
    ap.add_argument("--ws-test", type=int, default=512)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
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
