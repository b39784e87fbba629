"""Learned warm start for explicit dynamic relaxation of pressurised shells.

The problem family (no counterpart in the reference, which always starts from
the undeformed state): a closed level-5 icosphere shell (10,242 nodes, 20,480
faces) with a geometric imperfection, under a uniform external pressure held
constant, relaxed by the explicit Newmark solver with mass-proportional
damping until the relative residual ||f_ext - f_int - f_contact|| / ||f_ext||
(see shl_residual) falls below a tolerance.  Above the classical buckling
pressure (pressure / p_cl in [1.2, 3]) the sphere collapses: its equilibrium
is a buckled shape held by self-contact (linear, frictionless, so that the
equilibrium does not depend on the path; linked cells of 2h), and f_contact is
the static contact force of the current candidate list.

Eight inputs per problem:
  log(E1/E2) with E1 E2 = 1, nu12, G12 / sqrt(E1 E2), log(h/R),
  pressure / p_cl (p_cl = 2 E (h/R)^2 / sqrt(3 (1 - nu^2)) with E = sqrt(E1 E2),
  nu = sqrt(nu12 nu21)), and three coefficients c1..c3 of the imperfection
  w = 0.3 h (c1 Y20 + c2 Y21 + c3 Y31) along the unit normal, with the real
  spherical harmonics Y20 = (3 z^2 - 1) / 2, Y21 = sqrt(3) x z and
  Y31 = x (5 z^2 - 1) / 2 of the unit position.
The network (shl_mlp_*) maps the standardised inputs to the equilibrium
displacement field divided by h (3 x 10,242 values).  A warm start projects
the predicted field onto the leading principal directions of the training
fields (which removes the high-frequency error of the network's output: the
stiff membrane response turns even a small such error into a residual larger
than that of the zero start), runs a short phase of heavily damped steps (the
remaining stiff error decays, the smooth part hardly moves) and then relaxes
as the plain method does; the plain start remains the fallback when the warm
start does not converge.  With mass-proportional damping every underdamped
mode decays at the same rate, so the steps to a residual tolerance grow with
the logarithm of the initial residual, and that is what a warm start can save.
"""
import json
import time

import numpy as np

from . import lib as L

LEVEL = 5
DIMS = [8, 512, 512, 512, 512, 3 * 10242]
IMPERFECTION = 0.3        # amplitude of the imperfection in units of h
DAMPING = 1.0             # mass-proportional damping of the relaxation
DT = 4e-3                 # relaxation time step
CHECK_EVERY = 100         # steps between residual checks
S_RANGE = (1.2, 3.0)      # pressure / p_cl of the problems: the buckled (collapsed) regime


def harmonics(X):
    """Y20, Y21, Y31 (real, unnormalised) at the unit positions of X (n x 3)."""
    n = X / np.linalg.norm(X, axis=1, keepdims=True)
    x, z = n[:, 0], n[:, 2]
    return np.stack([(3 * z * z - 1) / 2, np.sqrt(3.0) * x * z, x * (5 * z * z - 1) / 2], 1), n


def sample_problems(n, seed, s_range=S_RANGE):
    """n problems from a seed (material, thickness, pressure, imperfection)."""
    rng = np.random.default_rng(seed)
    return {
        "ratio": np.exp(rng.uniform(np.log(0.2), np.log(5.0), n)),
        "nu": rng.uniform(0.25, 0.35, n),
        "g": rng.uniform(0.3, 0.45, n),
        "h": np.exp(rng.uniform(np.log(0.005), np.log(0.05), n)),
        "s": rng.uniform(s_range[0], s_range[1], n),
        "c": rng.standard_normal((n, 3)),
    }


def subset(problems, idx):
    return {k: v[idx] for k, v in problems.items()}


def features(pr):
    """Network inputs (n x 8, not yet standardised)."""
    return np.stack([np.log(pr["ratio"]), pr["nu"], pr["g"], np.log(pr["h"]), pr["s"], pr["c"][:, 0],
                     pr["c"][:, 1], pr["c"][:, 2]], 1).astype(np.float32)


def classical_pressure(e1, e2, nu12, h):
    E = np.sqrt(e1 * e2)
    nu = np.sqrt(nu12 * nu12 * e2 / e1)
    return 2 * E * h * h / np.sqrt(3 * (1 - nu * nu))


def build_batch(pr, precision=L.PREC_FP32, level=LEVEL, dt=DT, damping=DAMPING, contact=True):
    """One batch context over the problems; returns (batch, h per shell).
    contact: each shell with its own frictionless self-contact (linked cells of 2h)."""
    X0, T = L.icosphere(level)
    Y, nrm = harmonics(X0)
    P = X0[T]
    ext = (P.max(axis=1) - P.min(axis=1)).max(axis=1).mean()
    meshes, params, scale = [], [], []
    for k in range(len(pr["h"])):
        r, nu, g, h, s = (float(pr[q][k]) for q in ("ratio", "nu", "g", "h", "s"))
        e1, e2 = np.sqrt(r), 1.0 / np.sqrt(r)
        w = IMPERFECTION * h * (Y @ pr["c"][k])
        meshes.append((X0 + w[:, None] * nrm, T))
        params.append(L.default_params(shell_mass_density=1.0, shell_young_modulus=e1, shell_young_modulus2=e2,
                                       shell_poisson_ratio=nu, shell_shear_modulus=g * np.sqrt(e1 * e2),
                                       thickness=h, damping_alpha=damping, dt=dt,
                                       shell_shell_contact=L.CONTACT_LINEAR if contact else L.CONTACT_NONE,
                                       mu_s=0.0, mu_d=0.0, cell_size_mult=2 * h / ext, precision=precision))
        scale.append(s * classical_pressure(e1, e2, nu, h))
    return L.Batch(meshes, params, np.array(scale)), np.asarray(pr["h"], float)


def relax(batch, u_start, tol=1e-6, check_every=CHECK_EVERY, max_steps=40000, correct=True, smooth_steps=0,
          smooth_damping=200.0):
    """Explicit relaxation under the constant pressure (table value -1 times
    each shell's scale) from u_start (v = 0).  The residual is evaluated with
    FP64 forces; in an FP32 batch each check also refreshes the FP64 defect
    that the FP32 steps add (correct=True), without which FP32 relaxation
    stalls at the FP32 force error.  Returns a dict with the steps at which
    each shell's residual first fell below tol (-1 if never), the final
    residuals, the displacement at convergence and the wall time."""
    n = batch.n_shells
    flags = L.RESIDUAL_FP64 | (L.RESIDUAL_CORRECT if correct else L.RESIDUAL_CLEAR)
    if batch.params.shell_shell_contact != L.CONTACT_NONE:
        flags |= L.RESIDUAL_CONTACT
    t0 = time.perf_counter()
    batch.apply_initial_conditions(u_start, 0.0, -1.0)
    conv_step = np.full(n, -1, dtype=np.int64)
    u_conv = [None] * n
    steps = 0
    if smooth_steps:
        # heavily damped steps first: the stiff (membrane) error of a predicted field decays
        # within them, its smooth part hardly moves
        batch.scale_damping(smooth_damping / DAMPING)
        batch.step(smooth_steps, np.full(smooth_steps, -1.0))
        batch.scale_damping(1.0)
        steps = smooth_steps
    rel = batch.residual(-1.0, flags)
    table = np.full(check_every, -1.0)
    hist = [rel.copy()]
    for k in np.nonzero(rel < tol)[0]:
        conv_step[k] = steps
    if np.any(conv_step >= 0):
        u = batch.get_state()[0]
        for k in np.nonzero(conv_step >= 0)[0]:
            u_conv[k] = batch.split(u)[k].copy()
    while steps < max_steps and np.any(conv_step < 0):
        _, status = batch.step(check_every, table)
        steps += check_every
        rel = batch.residual(-1.0, flags)
        hist.append(rel.copy())
        new = np.nonzero((rel < tol) & (conv_step < 0))[0]
        if len(new):
            u = batch.get_state()[0]
            parts = batch.split(u)
            for k in new:
                conv_step[k] = steps
                u_conv[k] = parts[k].copy()
        if status >= 3 or not np.all(np.isfinite(rel)):
            break
    wall = time.perf_counter() - t0
    u = batch.get_state()[0]
    parts = batch.split(u)
    for k in range(n):
        if u_conv[k] is None:
            u_conv[k] = parts[k].copy()
    return {"conv_step": conv_step, "rel": rel, "u": u_conv, "wall_s": wall, "steps": steps,
            "history": np.array(hist)}


def drop_drift(u):
    """A displacement field without its mean translation (the drift of a free shell)."""
    x = np.asarray(u, np.float64).reshape(-1, 3)
    return (x - x.mean(0)).reshape(-1)


def standardizer(F):
    mu, sd = F.mean(0), F.std(0) + 1e-12
    return mu.astype(np.float32), sd.astype(np.float32)


def generate(problems, batch_size=512, precision=L.PREC_FP32, tol=5e-5, max_steps=10000, log=None, level=LEVEL,
             contact=True):
    """Equilibria of the problems by plain relaxation from zero, in batches.
    Returns (u_eq as n x 3V float64, conv_step, final residual, stats)."""
    n = len(problems["h"])
    U, steps, rels = [], [], []
    stats = {"wall_s": 0.0, "face_steps": 0.0, "setup_s": 0.0}
    for s in range(0, n, batch_size):
        idx = np.arange(s, min(n, s + batch_size))
        t0 = time.perf_counter()
        b, _ = build_batch(subset(problems, idx), precision=precision, level=level, contact=contact)
        stats["setup_s"] += time.perf_counter() - t0
        r = relax(b, np.zeros(3 * b.V), tol=tol, max_steps=max_steps)
        stats["wall_s"] += r["wall_s"]
        stats["face_steps"] += float(b.F) * r["steps"]
        U.extend(r["u"])
        steps.append(r["conv_step"])
        rels.append(r["rel"])
        b.close()
        if log:
            log("generated %d / %d (%.1f s, %d steps)" % (idx[-1] + 1, n, r["wall_s"], r["steps"]))
    return np.array(U), np.concatenate(steps), np.concatenate(rels), stats


def train_surrogate(F_train, U_train, h_train, iters=4000, batch=256, seed=0, lr0=1e-3, lr_final=1e-5, hidden=None):
    """Trains the network on standardised inputs and targets u / h (drift removed); returns (net, scaler, curve)."""
    mu, sd = standardizer(F_train)
    Xn = (F_train - mu) / sd
    Tn = (np.array([drop_drift(u) for u in U_train]) / h_train[:, None]).astype(np.float32)
    dims = DIMS if hidden is None else [DIMS[0]] + list(hidden) + [U_train.shape[1]]
    net = L.MLP(dims, max_batch=batch, seed=seed)
    net.set_dataset(Xn, Tn)
    curve = net.train(iters, batch, lr0=lr0, lr_final=lr_final, seed=seed, curve_every=max(1, iters // 50))
    return net, (mu, sd), curve


def predict(net, scaler, F, h):
    mu, sd = scaler
    Y = net.predict(((F - mu) / sd).astype(np.float32)).astype(np.float64)
    return Y * np.asarray(h)[:, None]


def pca_basis(T, k):
    """Mean and the k leading principal directions (rows) of the training
    fields T (n x 3V), from the eigenvectors of the n x n Gram matrix."""
    mean = T.mean(0)
    A = T - mean
    w, V = np.linalg.eigh(A @ A.T)
    idx = np.argsort(w)[::-1][:k]
    basis = (A.T @ V[:, idx]) / np.sqrt(np.maximum(w[idx], 1e-300))
    return mean, basis.T


def project(Y, mean, basis):
    """Projection of predicted fields onto the training fields' leading modes:
    it keeps what the network learned from the data and drops the
    high-frequency error of its output, which the stiff membrane response
    turns into a large residual."""
    Z = Y - mean
    return mean + (Z @ basis.T) @ basis


def solve(pr, U_start, level, precision, tol, max_steps, polish_tol=None, polish_max=None, smooth_steps=0,
          smooth_damping=200.0, contact=True):
    """Relaxation of a batch of problems from U_start (n x 3V).  With
    polish_tol, a second FP64 phase continues from the first phase's state
    (restarted at rest) down to polish_tol.  Returns per-shell steps to the
    final tolerance (-1: not reached), the final displacements, wall time and
    face-steps of each phase."""
    n = len(pr["h"])
    b, _ = build_batch(pr, precision=precision, level=level, contact=contact)
    F = b.F
    r = relax(b, np.asarray(U_start, np.float64).reshape(-1), tol=tol, max_steps=max_steps, smooth_steps=smooth_steps,
              smooth_damping=smooth_damping)
    b.close()
    out = {"steps": r["conv_step"].copy(), "u": r["u"], "wall_s": r["wall_s"],
           "r_first": float(np.median(r["history"][0])), "phases": [
        {"precision": "fp32" if precision == L.PREC_FP32 else "fp64", "steps": r["steps"], "wall_s": r["wall_s"],
         "face_steps_per_s": F * r["steps"] / r["wall_s"], "reached": int((r["conv_step"] >= 0).sum())}]}
    if polish_tol is None:
        return out
    b, _ = build_batch(pr, precision=L.PREC_FP64, level=level, contact=contact)
    r2 = relax(b, np.concatenate(r["u"]), tol=polish_tol, max_steps=polish_max)
    b.close()
    ok = (r["conv_step"] >= 0) & (r2["conv_step"] >= 0)
    out["steps"] = np.where(ok, r["conv_step"] + r2["conv_step"], -1)
    out["u"] = r2["u"]
    out["wall_s"] += r2["wall_s"]
    out["phases"].append({"precision": "fp64", "steps": r2["steps"], "wall_s": r2["wall_s"],
                          "face_steps_per_s": F * r2["steps"] / r2["wall_s"], "reached": int(ok.sum())})
    return out


def _stats(steps, mask):
    s = steps[mask]
    return {"median_steps": float(np.median(s)) if len(s) else None, "mean_steps": float(np.mean(s)) if len(s) else None}


def experiment(n_train=2048, n_test=256, seed=0, batch_size=512, train_iters=4000, gen_tol=5e-5, gen_max=10000,
               tol=1e-6, max_steps=15000, log=print, level=LEVEL, hidden=None, train_batch=256, s_range=S_RANGE,
               mixed=False, n_modes=32, smooth_steps=200, smooth_damping=200.0, contact=True):
    """The warm-start study.  Equilibria of n_train seeded problems by plain
    FP32 relaxation (FP64 defect correction) to gen_tol train the network;
    n_test held-out problems are then solved to the FP64 residual tol from
    zero (plain) and from the prediction (warm): in FP64, and (mixed=True) as
    FP32 relaxation to gen_tol followed by an FP64 polish.  Shells whose warm
    start does not converge fall back to the plain start (counted).  Returns
    a JSON-able summary."""
    t_all = time.perf_counter()
    out = {"level": level, "problems": {"train": n_train, "test": n_test, "seed": seed, "pressure_over_p_cl": s_range},
           "relaxation": {"dt": DT, "damping_alpha": DAMPING, "check_every": CHECK_EVERY, "tol": tol,
                          "fp32_tol": gen_tol}}
    pr = sample_problems(n_train + n_test, seed, s_range)
    F = features(pr)
    U, steps, rels, st = generate(subset(pr, np.arange(n_train)), batch_size, tol=gen_tol, max_steps=gen_max, log=log,
                                  level=level, contact=contact)
    ok = steps >= 0
    out["generation"] = {"converged": int(ok.sum()), "wall_s": st["wall_s"], "setup_s": st["setup_s"],
                         "fp32_face_steps_per_s": st["face_steps"] / st["wall_s"],
                         **_stats(steps, ok)}
    t1 = time.perf_counter()
    net, scaler, curve = train_surrogate(F[:n_train][ok], U[ok], pr["h"][:n_train][ok], iters=train_iters, seed=seed,
                                         hidden=hidden, batch=train_batch)
    out["training"] = {"samples": int(ok.sum()), "iters": train_iters, "batch": train_batch,
                       "wall_s": time.perf_counter() - t1, "loss_first": float(curve[0]), "loss_last": float(curve[-1])}
    test = subset(pr, np.arange(n_train, n_train + n_test))
    Ft, ht = F[n_train:], test["h"]
    tp = time.perf_counter()
    U_raw = predict(net, scaler, Ft, ht)
    pred_s = time.perf_counter() - tp
    Tn = np.array([drop_drift(u) for u in U[ok]]) / pr["h"][:n_train][ok][:, None]
    mean, basis = pca_basis(Tn, n_modes)
    U_pred = project(U_raw / ht[:, None], mean, basis) * ht[:, None]
    V3 = U_pred.shape[1]
    res = {}
    variants = [("fp64", dict(precision=L.PREC_FP64, tol=tol, max_steps=max_steps, contact=contact))]
    if mixed:
        variants.append(("fp32+fp64", dict(precision=L.PREC_FP32, tol=gen_tol, max_steps=gen_max, polish_tol=tol,
                                           polish_max=max_steps, contact=contact)))
    for name, kw in variants:
        plain = solve(test, np.zeros((n_test, V3)), level, **kw)
        warm = solve(test, U_pred, level, smooth_steps=smooth_steps, smooth_damping=smooth_damping, **kw)
        raw = solve(test, U_raw, level, **kw) if name == "fp64" else None
        base = plain["steps"] >= 0

        def summary(run):
            fb = run["steps"] < 0
            steps_fb = np.where(fb, np.where(base, plain["steps"] + max_steps, -1), run["steps"])
            dev = np.array([np.abs(drop_drift(run["u"][k]) - drop_drift(plain["u"][k])).max() for k in range(n_test)])
            ok2 = base & ~fb
            return {"converged": int((~fb).sum()), "fallbacks": int((fb & base).sum()), **_stats(steps_fb, base),
                    "wall_s": run["wall_s"] + pred_s, "phases": run["phases"], "first_residual_median":
                    run.get("r_first"),
                    "equilibrium_within_1e-4_of_plain": float(np.mean(dev[ok2] < 1e-4)) if ok2.any() else None,
                    "max_dev_from_plain": float(dev[ok2].max()) if ok2.any() else None}

        res[name] = {"plain": {"converged": int(base.sum()), **_stats(plain["steps"], base), "wall_s": plain["wall_s"],
                               "phases": plain["phases"]},
                     "warm": summary(warm)}
        if raw is not None:
            res[name]["warm_raw_prediction"] = summary(raw)
        res[name]["u_plain"] = plain["u"]
        if name == "fp64":
            err = np.array([np.abs(drop_drift(U_pred[k]) - drop_drift(plain["u"][k])).max() / ht[k]
                            for k in range(n_test)])
            res[name]["prediction_error_over_h"] = {"median": float(np.median(err[base])) if base.any() else None,
                                                    "max": float(err[base].max()) if base.any() else None}
        if log:
            log("%s: plain median %s, warm median %s" % (name, res[name]["plain"]["median_steps"],
                                                         res[name]["warm"]["median_steps"]))
    if mixed:
        ref = res["fp64"].pop("u_plain")
        mix = res["fp32+fp64"].pop("u_plain")
        dev = np.array([np.abs(drop_drift(mix[k]) - drop_drift(ref[k])).max() for k in range(n_test)])
        res["fp32+fp64"]["plain_vs_fp64_plain_within_1e-4"] = float(np.mean(dev < 1e-4))
    else:
        res["fp64"].pop("u_plain")
    out["test"] = res
    out["prediction_wall_s"] = pred_s
    out["total_wall_s"] = time.perf_counter() - t_all
    return out


def probe(n=32, seed=3, level=4, s_range=S_RANGE, contact=True, max_steps=80000, check_every=2000,
          precision=L.PREC_FP32, log=print):
    """Plain relaxation from zero of n seeded problems, the residual
    (quartiles over the shells) and the candidate pairs recorded every
    check_every steps: whether the problem family reaches equilibrium at all.
    Returns a JSON-able record."""
    pr = sample_problems(n, seed, s_range)
    b, _ = build_batch(pr, precision=precision, level=level, contact=contact)
    flags = L.RESIDUAL_FP64 | L.RESIDUAL_CORRECT | (L.RESIDUAL_CONTACT if contact else 0)
    t0 = time.perf_counter()
    b.apply_initial_conditions(np.zeros(3 * b.V), 0.0, -1.0)
    table = np.full(check_every, -1.0)
    conv = np.full(n, -1, dtype=np.int64)
    hist, steps, worst = [], 0, 0
    while steps < max_steps:
        _, st = b.step(check_every, table)
        worst = max(worst, int(st))
        steps += check_every
        rel = b.residual(-1.0, flags)
        conv[(rel < 1e-6) & (conv < 0)] = steps
        q = np.percentile(rel, [0, 25, 50, 75, 100])
        rec = {"steps": steps, "wall_s": time.perf_counter() - t0, "pairs": len(b.contact_state()["pairs"]),
               "converged": int((conv >= 0).sum()), "residual_quartiles": [float(x) for x in q], "status": int(st)}
        hist.append(rec)
        if log:
            log(json.dumps(rec))
        if st >= 3 or (conv >= 0).all():
            break
    b.close()
    return {"level": level, "shells": n, "seed": seed, "pressure_over_p_cl": list(s_range),
            "contact": "linear, frictionless, linked cells 2h" if contact else "none",
            "relaxation": {"dt": DT, "damping_alpha": DAMPING, "precision": "fp32 forces + fp64 defect correction"},
            "worst_status": worst, "converged": int((conv >= 0).sum()), "history": hist}


def _jsonable(o):
    if isinstance(o, dict):
        return {str(k): _jsonable(v) for k, v in o.items()}
    if isinstance(o, (list, tuple)):
        return [_jsonable(v) for v in o]
    if isinstance(o, np.generic):
        return o.item()
    return o


def main(argv=None):
    """python -m shell_gb300.warmstart --train N --test M --out study.json
    python -m shell_gb300.warmstart --probe --level 4 --shells 32 --out probe.json"""
    import argparse
    ap = argparse.ArgumentParser(description="learned warm start study (level-5 shells)")
    ap.add_argument("--train", type=int, default=3584)
    ap.add_argument("--test", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--train-iters", type=int, default=6000)
    ap.add_argument("--max-steps", type=int, default=15000)
    ap.add_argument("--out", default="warmstart_study.json")
    ap.add_argument("--probe", action="store_true", help="plain relaxation of the buckled family only")
    ap.add_argument("--level", type=int, default=LEVEL)
    ap.add_argument("--shells", type=int, default=32)
    a = ap.parse_args(argv)
    if a.probe:
        r = probe(n=a.shells, level=a.level, max_steps=a.max_steps, log=lambda m: print(m, flush=True))
        with open(a.out, "w") as f:
            json.dump(_jsonable(r), f, indent=1)
        return
    t0 = time.perf_counter()
    r = experiment(n_train=a.train, n_test=a.test, seed=a.seed, batch_size=512, train_iters=a.train_iters,
                   max_steps=a.max_steps, log=lambda m: print("[%.0f s] %s" % (time.perf_counter() - t0, m),
                                                              flush=True))
    with open(a.out, "w") as f:
        json.dump(_jsonable(r), f, indent=1)
    print(json.dumps(_jsonable(r)))


if __name__ == "__main__":
    main()
