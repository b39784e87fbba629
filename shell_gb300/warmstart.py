"""Learned warm start for explicit dynamic relaxation of pressurised shells.

The problem family (no counterpart in the reference, which always starts from
the undeformed state): a closed level-5 icosphere shell (10,242 nodes, 20,480
faces) with a geometric imperfection, under a uniform external pressure held
constant, relaxed by the explicit Newmark solver with mass-proportional
damping until the relative residual ||f_ext - f_int|| / ||f_ext|| (see
shl_residual) falls below a tolerance.

Eight inputs per problem:
  log(E1/E2) with E1 E2 = 1, nu12, G12 / sqrt(E1 E2), log(h/R),
  pressure / p_cl (p_cl = 2 E (h/R)^2 / sqrt(3 (1 - nu^2)) with E = sqrt(E1 E2),
  nu = sqrt(nu12 nu21)), and three coefficients c1..c3 of the imperfection
  w = 0.3 h (c1 Y20 + c2 Y21 + c3 Y31) along the unit normal, with the real
  spherical harmonics Y20 = (3 z^2 - 1) / 2, Y21 = sqrt(3) x z and
  Y31 = x (5 z^2 - 1) / 2 of the unit position.
The network (shl_mlp_*) maps the standardised inputs to the equilibrium
displacement field divided by h (3 x 10,242 values).  A warm start relaxes from
the predicted field instead of from zero; the plain start remains the
fallback when the warm start does not converge.
"""
import time

import numpy as np

from . import lib as L

LEVEL = 5
DIMS = [8, 512, 512, 512, 512, 3 * 10242]
IMPERFECTION = 0.3        # amplitude of the imperfection in units of h
DAMPING = 1.5             # mass-proportional damping of the relaxation
DT = 2e-3                 # relaxation time step
CHECK_EVERY = 50          # steps between residual checks


def harmonics(X):
    """Y20, Y21, Y31 (real, unnormalised) at the unit positions of X (n x 3)."""
    n = X / np.linalg.norm(X, axis=1, keepdims=True)
    x, z = n[:, 0], n[:, 2]
    return np.stack([(3 * z * z - 1) / 2, np.sqrt(3.0) * x * z, x * (5 * z * z - 1) / 2], 1), n


def sample_problems(n, seed, s_range=(0.3, 0.9)):
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


def build_batch(pr, precision=L.PREC_FP32, level=LEVEL, dt=DT, damping=DAMPING):
    """One batch context over the problems; returns (batch, h per shell)."""
    X0, T = L.icosphere(level)
    Y, nrm = harmonics(X0)
    meshes, params, scale = [], [], []
    for k in range(len(pr["h"])):
        r, nu, g, h, s = (float(pr[q][k]) for q in ("ratio", "nu", "g", "h", "s"))
        e1, e2 = np.sqrt(r), 1.0 / np.sqrt(r)
        w = IMPERFECTION * h * (Y @ pr["c"][k])
        meshes.append((X0 + w[:, None] * nrm, T))
        params.append(L.default_params(shell_mass_density=1.0, shell_young_modulus=e1, shell_young_modulus2=e2,
                                       shell_poisson_ratio=nu, shell_shear_modulus=g * np.sqrt(e1 * e2),
                                       thickness=h, damping_alpha=damping, dt=dt,
                                       shell_shell_contact=L.CONTACT_NONE, precision=precision))
        scale.append(s * classical_pressure(e1, e2, nu, h))
    return L.Batch(meshes, params, np.array(scale)), np.asarray(pr["h"], float)


def relax(batch, u_start, tol=1e-6, check_every=CHECK_EVERY, max_steps=40000, correct=True):
    """Explicit relaxation under the constant pressure (table value -1 times
    each shell's scale) from u_start (v = 0).  The residual is evaluated with
    FP64 forces; in an FP32 batch each check also refreshes the FP64 defect
    that the FP32 steps add (correct=True), without which FP32 relaxation
    stalls at the FP32 force error.  Returns a dict with the steps at which
    each shell's residual first fell below tol (-1 if never), the final
    residuals, the displacement at convergence and the wall time."""
    n = batch.n_shells
    flags = L.RESIDUAL_FP64 | (L.RESIDUAL_CORRECT if correct else L.RESIDUAL_CLEAR)
    t0 = time.perf_counter()
    batch.apply_initial_conditions(u_start, 0.0, -1.0)
    conv_step = np.full(n, -1, dtype=np.int64)
    u_conv = [None] * n
    rel = batch.residual(-1.0, flags)
    steps = 0
    table = np.full(check_every, -1.0)
    hist = [rel.copy()]
    for k in np.nonzero(rel < tol)[0]:
        conv_step[k] = 0
    if np.any(conv_step == 0):
        u = batch.get_state()[0]
        for k in np.nonzero(conv_step == 0)[0]:
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


def standardizer(F):
    mu, sd = F.mean(0), F.std(0) + 1e-12
    return mu.astype(np.float32), sd.astype(np.float32)


def generate(problems, batch_size=512, precision=L.PREC_FP32, tol=1e-6, max_steps=40000, log=None, level=LEVEL):
    """Equilibria of the problems by plain relaxation from zero, in batches.
    Returns (u_eq as n x 3V float64, conv_step, final residual, stats)."""
    n = len(problems["h"])
    U, steps, rels = [], [], []
    stats = {"wall_s": 0.0, "face_steps": 0.0, "setup_s": 0.0}
    for s in range(0, n, batch_size):
        idx = np.arange(s, min(n, s + batch_size))
        t0 = time.perf_counter()
        b, _ = build_batch(subset(problems, idx), precision=precision, level=level)
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
    """Trains the network on standardised inputs and targets u / h; returns (net, scaler, loss curve)."""
    mu, sd = standardizer(F_train)
    Xn = (F_train - mu) / sd
    Tn = (U_train / h_train[:, None]).astype(np.float32)
    dims = DIMS if hidden is None else [DIMS[0]] + list(hidden) + [U_train.shape[1]]
    net = L.MLP(dims, max_batch=batch, seed=seed)
    net.set_dataset(Xn, Tn)
    curve = net.train(iters, batch, lr0=lr0, lr_final=lr_final, seed=seed, curve_every=max(1, iters // 50))
    return net, (mu, sd), curve


def predict(net, scaler, F, h):
    mu, sd = scaler
    Y = net.predict(((F - mu) / sd).astype(np.float32)).astype(np.float64)
    return Y * np.asarray(h)[:, None]


def experiment(n_train=3584, n_test=512, seed=0, batch_size=512, train_iters=4000, tol=1e-6, max_steps=40000,
               fp64_check=True, log=print, level=LEVEL, hidden=None, train_batch=256):
    """The whole warm-start study: equilibria of n_train + n_test seeded
    problems by plain FP32 relaxation, the network trained on the first
    n_train, then the n_test held-out problems relaxed from zero and from the
    prediction (FP32 forces), with the plain start as fallback; optionally the
    held-out problems relaxed in FP64 from zero as the accuracy reference and
    for the FP64 face-steps/s.  Returns a JSON-able summary."""
    out = {}
    pr = sample_problems(n_train + n_test, seed)
    F = features(pr)
    t0 = time.perf_counter()
    U, steps, rels, st = generate(subset(pr, np.arange(n_train)), batch_size, tol=tol, max_steps=max_steps, log=log,
                                  level=level)
    ok = steps >= 0
    out["generation"] = {"problems": n_train, "converged": int(ok.sum()), "wall_s": st["wall_s"],
                         "setup_s": st["setup_s"], "face_steps_per_s": st["face_steps"] / st["wall_s"],
                         "median_steps": float(np.median(steps[ok])) if ok.any() else None}
    t1 = time.perf_counter()
    net, scaler, curve = train_surrogate(F[:n_train][ok], U[ok], pr["h"][:n_train][ok], iters=train_iters, seed=seed,
                                         hidden=hidden, batch=train_batch)
    out["training"] = {"samples": int(ok.sum()), "iters": train_iters, "wall_s": time.perf_counter() - t1,
                       "loss_first": float(curve[0]), "loss_last": float(curve[-1])}
    test = subset(pr, np.arange(n_train, n_train + n_test))
    Ft, ht = F[n_train:], test["h"]
    # plain start
    b, _ = build_batch(test, level=level)
    plain = relax(b, np.zeros(3 * b.V), tol=tol, max_steps=max_steps)
    F_faces = b.F
    b.close()
    # warm start from the prediction
    tp = time.perf_counter()
    U_pred = predict(net, scaler, Ft, ht)
    pred_s = time.perf_counter() - tp
    b, _ = build_batch(test, level=level)
    warm = relax(b, U_pred.reshape(-1), tol=tol, max_steps=max_steps)
    b.close()
    # fallback: shells whose warm start did not converge restart from zero (the plain result)
    fb = warm["conv_step"] < 0
    warm_steps = np.where(fb, max_steps + np.maximum(plain["conv_step"], 0), warm["conv_step"])
    both = (plain["conv_step"] >= 0)
    out["test"] = {
        "problems": n_test, "faces_per_batch": int(F_faces), "prediction_s": pred_s,
        "plain": {"converged": int(both.sum()), "median_steps": float(np.median(plain["conv_step"][both])),
                  "mean_steps": float(np.mean(plain["conv_step"][both])), "wall_s_all": plain["wall_s"],
                  "steps_all": plain["steps"]},
        "warm": {"converged": int((~fb).sum()), "fallbacks": int(fb.sum()),
                 "median_steps": float(np.median(warm_steps[both])), "mean_steps": float(np.mean(warm_steps[both])),
                 "wall_s_all": warm["wall_s"] + pred_s, "steps_all": warm["steps"]},
        "prediction_error_vs_plain_eq": float(np.median([np.abs(U_pred[k] - plain["u"][k]).max() / ht[k]
                                                          for k in range(n_test)])),
    }
    if fp64_check:
        b, _ = build_batch(test, precision=L.PREC_FP64, level=level)
        ref = relax(b, np.zeros(3 * b.V), tol=tol, max_steps=max_steps)
        b.close()
        okr = ref["conv_step"] >= 0
        d_plain = np.array([np.abs(plain["u"][k] - ref["u"][k]).max() for k in range(n_test)])
        d_warm = np.array([np.abs(warm["u"][k] - ref["u"][k]).max() for k in range(n_test)])
        out["fp64_reference"] = {
            "converged": int(okr.sum()), "wall_s_all": ref["wall_s"], "steps_all": ref["steps"],
            "face_steps_per_s": F_faces * ref["steps"] / ref["wall_s"],
            "fp32_face_steps_per_s": F_faces * plain["steps"] / plain["wall_s"],
            "plain_fp32_within_1e-4": float(np.mean(d_plain[okr] < 1e-4)),
            "warm_fp32_within_1e-4": float(np.mean(d_warm[okr] < 1e-4)),
            "max_dev_plain": float(d_plain[okr].max()) if okr.any() else None,
        }
    out["total_wall_s"] = time.perf_counter() - t0
    return out
