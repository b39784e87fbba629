"""Synthetic workloads of the benchmark and the profiling runs (no datasets:
generated icospheres and seeded perturbations).

The single-shell configuration: an icosphere of the given level, orthotropic
Koiter shell E1 = 1, E2 = 0.5, nu12 = 0.3, G12 = 0.35, h/R = 0.01, density 1,
Rayleigh damping 0.05, dt = 1e-4, a seeded Gaussian normal imperfection of
amplitude 1e-3 R, self-contact with Coulomb friction mu = 0.3 and linked cells
of 2h, and an external pressure ramped from 0 to 2 p_cl over 20,000 steps.
"""
import numpy as np

E1, E2, NU12, G12, H, RHO, ALPHA, DT = 1.0, 0.5, 0.3, 0.35, 0.01, 1.0, 0.05, 1e-4
RAMP_STEPS, RAMP_FACTOR, AMPL, SEED, MU = 20000, 2.0, 1e-3, 0, 0.3


def classical_pressure():
    """p_cl = 2 E_eff (h/R)^2 / sqrt(3 (1 - nu_eff^2)), E_eff = sqrt(E1 E2), nu_eff = sqrt(nu12 nu21)."""
    E = np.sqrt(E1 * E2)
    nu = np.sqrt(NU12 * NU12 * E2 / E1)
    return 2 * E * H * H / np.sqrt(3 * (1 - nu * nu))


def workload(api, level, contact=None):
    """Mesh, parameters and initial displacement of the single-shell workload.

    `api` provides icosphere, default_params, gaussian_normal_imperfection and
    the CONTACT_* constants: the library's binding (shell_gb300.lib) or the
    oracle's own input generators (oracle.inputs), which give the same inputs
    bit for bit without loading the CUDA library.  Every parameter whose
    default differs between the two is set here."""
    X, T = api.icosphere(level)
    P = X[T]
    cell_mult = 2 * H / (P.max(axis=1) - P.min(axis=1)).max(axis=1).mean()
    p = api.default_params(shell_mass_density=RHO, shell_young_modulus=E1, shell_young_modulus2=E2,
                           shell_poisson_ratio=NU12, shell_shear_modulus=G12, thickness=H, damping_alpha=ALPHA,
                           dt=DT, shell_shell_contact=api.CONTACT_LINEAR if contact is None else contact, mu_s=MU,
                           mu_d=MU, cell_size_mult=cell_mult, adapt_dt_every=0, rel_loc_err_min=5e-5,
                           rel_loc_err_max=5e-4, shell_cavity_contact=0)
    u0 = api.gaussian_normal_imperfection(X, AMPL, SEED).reshape(-1)
    return X, T, p, u0


def pressure(step):
    """p(t) at the end of step `step` (1-based): -s p_cl t / T."""
    return -RAMP_FACTOR * classical_pressure() * np.asarray(step, dtype=np.float64) / RAMP_STEPS


def squashed_state(X, s=0.0042, seed=0):
    """The sphere flattened to a double layer (gap about 2 s |z|) with 2e-5
    seeded noise: every face has contact candidates on the other layer."""
    rng = np.random.default_rng(seed)
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    return (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)


def ensemble_workload(L, n_shells=256, seed=0):
    """256 shells, levels uniform over 3/4/5, per-shell parameters from a seed:
    E1/E2 log-uniform in [0.2, 5] (E1 E2 = 1), h/R log-uniform in [0.005, 0.05],
    pressure ramp end uniform in [1.2, 3] p_cl of the shell, imperfection
    amplitude log-uniform in [1e-4, 1e-2] R; FP32 element forces, FP64 state;
    each shell with its own self-contact (linear, Coulomb friction mu = 0.3,
    linked cells of 2h: contact gaps in FP64)."""
    rng = np.random.default_rng(seed)
    meshes = {lv: L.icosphere(lv) for lv in (3, 4, 5)}
    ext = {}
    for lv, (X, T) in meshes.items():
        P = X[T]
        ext[lv] = (P.max(axis=1) - P.min(axis=1)).max(axis=1).mean()
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
                                       damping_alpha=ALPHA, dt=DT, shell_shell_contact=L.CONTACT_LINEAR, mu_s=MU,
                                       mu_d=MU, cell_size_mult=2 * h / ext[lv], precision=L.PREC_FP32))
        shells.append((X, T))
        scale.append(s * p_cl)
        u0.append(L.gaussian_normal_imperfection(X, amp, seed * 100000 + k).reshape(-1))
    return shells, params, np.array(scale), np.concatenate(u0)
