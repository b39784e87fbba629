"""Inputs of the oracle runs, generated without the CUDA library.

TEST INFRASTRUCTURE ONLY.  The CPU reference arm of `bench.py` and the tests
build the mesh, the parameters and the seeded imperfection here, so that a
CPU-only run loads no part of libshl_gb300.so.  The definitions are the
workloads', restated on their own:

  icosphere(level)  the closed icosphere as the reference's OFF files hold it
                    (icosasphere3.off / icosasphere4.off are reproduced byte for
                    byte): the 12 normalised icosahedron vertices, 20 faces, and
                    per refinement face (a, b, c) -> (a, ab, ca), (b, bc, ab),
                    (c, ca, bc), (ab, bc, ca), each edge midpoint appended on
                    first use and pushed to the unit sphere; written with "%g"
                    and read back, as the reference reads an OFF file
                    (shell.C:167).
  gaussian_normal_imperfection(X, A, seed)
                    u_i = A g_i x_i / |x_i| with g_i ~ N(0, 1): Philox-4x32-10
                    (Salmon et al., SC'11; key = seed, counter = (node id,
                    0x5348454C, 0, 0)), two 53-bit uniforms (u + 1/2) / 2^53 and
                    the Box-Muller map sqrt(-2 log u1) cos(2 pi u2), with the C
                    library's log and cos (Python's math module calls them).
  default_params(**kw)
                    the parameter defaults of the ShellSystem constructor and
                    set_parameters (ShellSystem.C:23-142, 170-318).
"""
import math

import numpy as np


def icosphere_text(level):
    """OFF text of the level-`level` icosphere."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    base = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
            (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = []

    def unit(x, y, z):
        n = math.sqrt(x * x + y * y + z * z)
        verts.append((x / n, y / n, z / n))
        return len(verts) - 1

    for p in base:
        unit(float(p[0]), float(p[1]), float(p[2]))
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        mids = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            m = mids.get(key)
            if m is None:
                pa, pb = verts[a], verts[b]
                m = unit((pa[0] + pb[0]) / 2, (pa[1] + pb[1]) / 2, (pa[2] + pb[2]) / 2)
                mids[key] = m
            return m

        refined = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            refined += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = refined
    lines = ["OFF", "%d %d 0" % (len(verts), len(faces))]
    lines += ["%g %g %g" % v for v in verts]
    lines += ["3 %d %d %d" % f for f in faces]
    return "\n".join(lines) + "\n"


def parse_off(text):
    tok = text.split()
    if tok[0] != "OFF":
        raise ValueError("not an OFF file")
    nv, nf = int(tok[1]), int(tok[2])
    X = np.array([float(x) for x in tok[4:4 + 3 * nv]], dtype=np.float64).reshape(nv, 3)
    F = np.array([int(x) for x in tok[4 + 3 * nv:4 + 3 * nv + 4 * nf]], dtype=np.int64).reshape(nf, 4)
    if (F[:, 0] != 3).any():
        raise ValueError("OFF face is not a triangle")
    return X, F[:, 1:].astype(np.uint32)


def icosphere(level):
    """Node positions (V, 3) and faces (F, 3) as read back from the OFF text."""
    return parse_off(icosphere_text(level))


_M0, _M1, _W0, _W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Ten Philox rounds on uint64 arrays holding 32-bit words."""
    k0, k1 = np.uint64(k0), np.uint64(k1)
    mask = np.uint64(_MASK)
    for _ in range(10):
        p0 = np.uint64(_M0) * c0
        p1 = np.uint64(_M1) * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + np.uint64(_W0)) & mask
        k1 = (k1 + np.uint64(_W1)) & mask
    return c0, c1, c2, c3


def gaussian_normal_imperfection(X, amplitude, seed):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    c0 = np.arange(n, dtype=np.uint64)
    c1 = np.full(n, 0x5348454C, dtype=np.uint64)
    z = np.zeros(n, dtype=np.uint64)
    r0, r1, r2, r3 = philox4x32_10(c0, c1, z, z.copy(), seed & _MASK, (seed >> 32) & _MASK)
    two53 = 9007199254740992.0
    m1 = ((r0 >> np.uint64(5)) << np.uint64(26)) | (r1 >> np.uint64(6))
    m2 = ((r2 >> np.uint64(5)) << np.uint64(26)) | (r3 >> np.uint64(6))
    u1 = (m1.astype(np.float64) + 0.5) / two53
    u2 = (m2.astype(np.float64) + 0.5) / two53
    u = np.zeros_like(X)
    for i in range(n):
        g = math.sqrt(-2.0 * math.log(float(u1[i]))) * math.cos(2.0 * math.pi * float(u2[i]))
        x, y, zz = (float(c) for c in X[i])
        r = math.sqrt(x * x + y * y + zz * zz)
        if r > 0:
            u[i] = (amplitude * g * x / r, amplitude * g * y / r, amplitude * g * zz / r)
    return u


# constants of shl.h (the ABI the oracle implements)
CONTACT_LINEAR, CONTACT_SMOOTH, CONTACT_NONE = 0, 1, 2
CS_LOCAL = 0
PREC_FP64, PREC_FP32 = 0, 1
CAVITY_ELLIPSOID = 2

# ShellSystem constructor (ShellSystem.C:23-142) and set_parameters defaults
# (MAKE_FUNCTION / STR_PARSE / MAKE_PARSE, ShellSystem.C:176-318)
REFERENCE_DEFAULTS = dict(
    shell_mass_density=1e3, shell_young_modulus=1e9, shell_young_modulus2=1e9, shell_poisson_ratio=1.0 / 3.0,
    shell_shear_modulus=0.0, bulk_modulus=0.0, memb_stiff_mult=1.0, bend_stiff_mult=1.0, thickness=1e-3,
    damping_alpha=0.0, damping_beta=0.0, damping_gamma=0.0, pressure=0.0, pressure_base=CS_LOCAL, pressure_dir=2,
    shell_shell_contact=CONTACT_NONE, mu_s=0.0, mu_d=0.0, self_damping=0.0, self_friction_damping=0.0,
    fric_stiff_mult=1.0, friction_stop_velocity=0.03, static_friction_tol=0.1, cell_size_mult=4.0, cell_margin=0.02,
    neighbor_margin=0.4, dt=1e-6, newmark_beta=0.25, newmark_gamma=0.5, compat_zero_pressure=0,
    precision=PREC_FP64, stop_on_problem=0, adapt_dt_every=1, dt_min=0.0, dt_max=0.0, rel_loc_err_min=3e-5,
    rel_loc_err_max=3e-4, shell_cavity_contact=1, cavity=CAVITY_ELLIPSOID, Rx=0.1005, Ry=0.1005, Rz=0.1005,
    mu_s_cavity=0.0, mu_d_cavity=0.0, cavity_damping=0.0, cavity_friction_damping=0.0)


def default_params(**kw):
    """shl_params (the structure the oracle takes) with the reference's defaults."""
    from shell_gb300.abi import ShlParams

    p = ShlParams()
    for k, v in REFERENCE_DEFAULTS.items():
        setattr(p, k, v)
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p
