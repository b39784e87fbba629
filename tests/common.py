"""Shared parameter sets of the tests (synthetic icosphere shells)."""
import numpy as np

from shell_gb300 import lib as L


def physics_params(contact=True, **kw):
    """Orthotropic shell of the benchmark workloads (E1=1, E2=0.5, nu12=0.3,
    G12=0.35, h/R=0.01, density 1, Rayleigh damping 0.05, dt=1e-4, linear
    self-contact with Coulomb friction mu=0.3)."""
    p = dict(shell_mass_density=1.0, shell_young_modulus=1.0, shell_young_modulus2=0.5, shell_poisson_ratio=0.3,
             shell_shear_modulus=0.35, thickness=0.01, damping_alpha=0.05, dt=1e-4,
             shell_shell_contact=L.CONTACT_LINEAR if contact else L.CONTACT_NONE, mu_s=0.3, mu_d=0.3,
             cell_size_mult=1.0)
    p.update(kw)
    return L.default_params(**p)


def classical_pressure(E1=1.0, E2=0.5, nu12=0.3, h=0.01, R=1.0):
    """p_cl = 2 E_eff (h/R)^2 / sqrt(3 (1 - nu_eff^2)), E_eff = sqrt(E1 E2),
    nu_eff = sqrt(nu12 nu21), nu21 = nu12 E2/E1."""
    E = np.sqrt(E1 * E2)
    nu = np.sqrt(nu12 * nu12 * E2 / E1)
    return 2 * E * (h / R) ** 2 / np.sqrt(3 * (1 - nu * nu))


def cell_size_mult_for(X, T, h):
    """cell_size_mult such that the linked cells are 2h wide at the reference
    configuration (cell_size_mult * avg_elem_size = 2h)."""
    P = X[T]
    ext = (P.max(axis=1) - P.min(axis=1)).max(axis=1)
    return 2 * h / ext.mean()


def folded_state(X, rng, amplitude=0.05):
    """A smooth large displacement that pushes the upper cap down onto the
    lower half (creates near-contacts without interpenetration)."""
    z = X[:, 2]
    u = np.zeros_like(X)
    u[:, 2] = -amplitude * np.clip(z, 0, None) ** 2
    u += 1e-4 * rng.standard_normal(X.shape)
    return u.reshape(-1)


def midpoint_refine(X, T, project=True):
    """Each triangle split into four at its edge midpoints (new nodes projected
    onto the unit sphere when `project`)."""
    X = [tuple(x) for x in np.asarray(X, float)]
    cache = {}

    def mid(a, b):
        k = (min(a, b), max(a, b))
        if k not in cache:
            m = (np.asarray(X[a]) + np.asarray(X[b])) / 2
            if project:
                m = m / np.linalg.norm(m)
            cache[k] = len(X)
            X.append(tuple(m))
        return cache[k]

    out = []
    for a, b, c in np.asarray(T, int):
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        out += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    return np.array(X), np.array(out, dtype=np.uint32)


def flipped_sphere(level=1):
    """An icosphere of level 2 with one edge flipped (two vertices of valence
    7, two more of valence 5), refined `level` times: patches of valence 5, 6
    and 7 (13 patch nodes)."""
    X, T = L.icosphere(2)
    T = np.array(T, dtype=np.int64)
    val = np.bincount(T.ravel())
    faces_of = {}
    for f, t in enumerate(T):
        for k in range(3):
            faces_of[(int(t[k]), int(t[(k + 1) % 3]))] = f
    for f, t in enumerate(T):
        for k in range(3):
            p, q = int(t[k]), int(t[(k + 1) % 3])
            r = int(t[(k + 2) % 3])
            g = faces_of[(q, p)]
            s = [int(x) for x in T[g] if x != p and x != q][0]
            if val[p] == val[q] == val[r] == val[s] == 6:
                # (p, q, r) and (q, p, s) -> (r, s, q) and (s, r, p)
                T[f] = (r, s, q)
                T[g] = (s, r, p)
                for _ in range(level):
                    X, T = midpoint_refine(X, T)
                return np.ascontiguousarray(X, dtype=np.float64), np.ascontiguousarray(T, dtype=np.uint32)
    raise AssertionError("no flippable edge")
