"""CPU tests of the oracle: pinned against the reference's fixtures and against
known answers (the reference ships no force or state vectors)."""
import hashlib
import json
import os

import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import classical_pressure, physics_params

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def mesh3(built):
    return L.icosphere(3)


def test_fp_contract_off(built):
    assert O.fp_contract_off(), "oracle must be built with -ffp-contract=off"


@pytest.mark.parametrize("level", [3, 4])
def test_icosphere_matches_reference_off(built, level):
    """The generator reproduces icosasphere3.off / icosasphere4.off byte for byte."""
    g = json.load(open(os.path.join(GOLDEN, "icosphere_off.json")))[str(level)]
    text = L.icosphere_off(level)
    lines = text.splitlines()
    for i, line in g["samples"].items():
        assert lines[int(i)] == line
    assert len(text.encode()) == g["bytes"]
    assert hashlib.sha256(text.encode()).hexdigest() == g["sha256"]
    X, T = L.icosphere(level)
    assert X.shape == (g["n_nodes"], 3) and T.shape == (g["n_faces"], 3)


def _loop_subdivide(F, val):
    """One Loop step of a scalar field on a closed mesh (Loop's beta(N))."""
    nbr = [set() for _ in range(len(val))]
    opp = {}
    for a, b, c in F:
        nbr[a] |= {b, c}; nbr[b] |= {a, c}; nbr[c] |= {a, b}
        for x, y, z in ((a, b, c), (b, c, a), (c, a, b)):
            opp.setdefault((min(x, y), max(x, y)), []).append(z)
    new = []
    for i in range(len(val)):
        N = len(nbr[i]); t = 3 / 8 + 0.25 * np.cos(2 * np.pi / N); beta = (5 / 8 - t * t) / N
        new.append((1 - N * beta) * val[i] + beta * sum(val[j] for j in nbr[i]))
    cache = {}

    def mid(i, j):
        k = (min(i, j), max(i, j))
        if k not in cache:
            r, s = opp[k]
            new.append(3 / 8 * (val[i] + val[j]) + 1 / 8 * (val[r] + val[s]))
            cache[k] = len(new) - 1
        return cache[k]

    NF = []
    for a, b, c in F:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        NF += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    return NF, new


def test_basis_equals_loop_limit(mesh3):
    """Basis values at dyadic points equal the Loop limit of the subdivided
    control net (regular patches anywhere; valence-5 patches in the middle
    sub-triangle, which holds the quadrature point)."""
    X, T = mesh3
    o = O.Oracle(X, T, physics_params(contact=False), threads=1)
    rng = np.random.default_rng(1)
    val = list(rng.standard_normal(len(X)))
    F0 = [tuple(int(x) for x in t) for t in T]
    K = 3
    Fk, vk = F0, val
    for _ in range(K):
        Fk, vk = _loop_subdivide(Fk, vk)
    nbrK = [set() for _ in range(len(vk))]
    for a, b, c in Fk:
        nbrK[a] |= {b, c}; nbrK[b] |= {a, c}; nbrK[c] |= {a, b}

    def limit(vid):
        N = len(nbrK[vid]); t = 3 / 8 + 0.25 * np.cos(2 * np.pi / N); beta = (5 / 8 - t * t) / N
        chi = 1 / (3 / (8 * beta) + N)
        return (1 - N * chi) * vk[vid] + chi * sum(vk[j] for j in nbrK[vid])

    def child_vertex(e, v, w):
        idx, corners = e, [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]
        for _ in range(K):
            A, B, C = corners
            ab = ((A[0] + B[0]) / 2, (A[1] + B[1]) / 2); bc = ((B[0] + C[0]) / 2, (B[1] + C[1]) / 2)
            ca = ((C[0] + A[0]) / 2, (C[1] + A[1]) / 2)
            kids = [(A, ab, ca), (B, bc, ab), (C, ca, bc), (ab, bc, ca)]
            for ci, ((x0, y0), (x1, y1), (x2, y2)) in enumerate(kids):
                det = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0)
                l1 = ((v - x0) * (y2 - y0) - (x2 - x0) * (w - y0)) / det
                l2 = ((x1 - x0) * (w - y0) - (v - x0) * (y1 - y0)) / det
                if l1 >= -1e-12 and l2 >= -1e-12 and l1 + l2 <= 1 + 1e-12:
                    idx, corners = idx * 4 + ci, list(kids[ci]); break
        for q, vid in zip(corners, Fk[idx]):
            if abs(q[0] - v) < 1e-12 and abs(q[1] - w) < 1e-12:
                return vid
        raise AssertionError("no vertex at (%g, %g)" % (v, w))

    valence = np.bincount(T.ravel())
    irr = [e for e in range(len(T)) if (valence[T[e]] != 6).any()]
    assert len(irr) == 60
    val = np.array(val)
    reg_pts = [(0.25, 0.25), (0.375, 0.25), (0.125, 0.5), (0.5, 0.5), (0.625, 0.125), (0.0, 0.0), (0.125, 0.75)]
    mid_pts = [(0.375, 0.25), (0.25, 0.375), (0.375, 0.375), (0.375, 0.125 + 0.25)]
    worst = 0.0
    for e in list(range(0, len(T), 61)) + irr[::3]:
        ids = o.patch(e)
        for v, w in (mid_pts if e in irr else reg_pts):
            B = o.basis_at(e, v, w)
            worst = max(worst, abs(B[:, 0] @ val[ids] - limit(child_vertex(e, v, w))))
    assert worst < 1e-13


def test_basis_derivatives_by_finite_differences(mesh3):
    X, T = mesh3
    o = O.Oracle(X, T, physics_params(contact=False), threads=1)
    valence = np.bincount(T.ravel())
    irr = [e for e in range(len(T)) if (valence[T[e]] != 6).any()]
    h = 1e-5
    for e in (0, 100, irr[0], irr[7]):
        v, w = 1 / 3, 1 / 3
        B = o.basis_at(e, v, w)
        fd_v = (o.basis_at(e, v + h, w) - o.basis_at(e, v - h, w)) / (2 * h)
        fd_w = (o.basis_at(e, v, w + h) - o.basis_at(e, v, w - h)) / (2 * h)
        assert np.abs(fd_v[:, 0] - B[:, 1]).max() < 1e-8
        assert np.abs(fd_w[:, 0] - B[:, 2]).max() < 1e-8
        assert np.abs(fd_v[:, 1] - B[:, 3]).max() < 1e-7
        assert np.abs(fd_w[:, 2] - B[:, 4]).max() < 1e-7
        assert np.abs(fd_w[:, 1] - B[:, 5]).max() < 1e-7
        # partition of unity and linear precision in the parameter plane
        assert abs(B[:, 0].sum() - 1) < 1e-14
        assert np.abs(B[:, 1:].sum(axis=0)).max() < 1e-13


def test_force_is_energy_gradient(mesh3):
    X, T = mesh3
    o = O.Oracle(X, T, physics_params(contact=False), threads=1)
    rng = np.random.default_rng(0)
    u = 0.01 * rng.standard_normal(3 * len(X))
    z = np.zeros_like(u)
    f = o.eval_forces(u, z, 0.0)[0]

    def energy(uu):
        e = o.eval_forces(uu, z, 0.0)[2]
        return e["Etens"] + e["Ebend"]

    h = 1e-6
    for d in rng.choice(len(u), 6, replace=False):
        up, um = u.copy(), u.copy()
        up[d] += h; um[d] -= h
        g = (energy(up) - energy(um)) / (2 * h)
        assert abs(f[d] + g) <= 1e-7 * abs(g)


def test_rigid_motion_gives_no_force(mesh3):
    X, T = mesh3
    o = O.Oracle(X, T, physics_params(contact=False), threads=1)
    z = np.zeros(3 * len(X))
    th = 0.4
    R = np.array([[np.cos(th), 0, np.sin(th)], [0, 1, 0], [-np.sin(th), 0, np.cos(th)]])
    for u in (np.tile([0.1, -0.2, 0.3], len(X)), (X @ R.T - X).reshape(-1)):
        f, _, e, _ = o.eval_forces(u, z, 0.0)
        assert np.abs(f).max() < 1e-15 and abs(e["Etens"]) < 1e-20 and abs(e["Ebend"]) < 1e-20


def test_pressure_resultant(mesh3):
    """Uniform pressure on a closed surface has (nearly) zero resultant and
    does work p * dV: f . u_radial = -p dV for a uniform radial expansion."""
    X, T = mesh3
    o = O.Oracle(X, T, physics_params(contact=False), threads=1)
    z = np.zeros(3 * len(X))
    f0 = o.eval_forces(z, z, 0.0)[0]
    f1 = o.eval_forces(z, z, -1.0)[0]
    fp = (f1 - f0).reshape(-1, 3)
    assert np.abs(fp.sum(axis=0)).max() < 1e-12
    radial = (X / np.linalg.norm(X, axis=1)[:, None])
    work = (fp * radial).sum()
    assert work < 0 and abs(work + 4 * np.pi) < 0.1 * 4 * np.pi


def test_mass_lumping_total(mesh3):
    X, T = mesh3
    p = physics_params(contact=False, shell_mass_density=2.0, thickness=0.01)
    o = O.Oracle(X, T, p, threads=1)
    Minv, C = o.mass_damping()
    total = (1.0 / Minv).reshape(-1, 3)[:, 0].sum()
    o.eval_forces(np.zeros(3 * len(X)), np.zeros(3 * len(X)), 0.0)
    area = o.element_fields()["area"].sum()
    assert abs(total - 2.0 * 0.01 * area) < 1e-10
    assert np.allclose(C, 0.05 * (1.0 / Minv))


def test_segment_segment_bruteforce(built):
    rng = np.random.default_rng(2)
    s = np.linspace(0, 1, 401)
    for _ in range(60):
        p = rng.standard_normal((4, 3))
        if rng.random() < 0.2:
            p[3] = p[2] + 0.7 * (p[1] - p[0])  # parallel
        dv, st = O.segment_segment(*p)
        a = p[0] + s[:, None] * (p[1] - p[0])
        b = p[2] + s[:, None] * (p[3] - p[2])
        d = np.linalg.norm(a[:, None, :] - b[None, :, :], axis=2).min()
        assert np.linalg.norm(dv) <= d + 1e-12
        assert np.linalg.norm(dv) >= d - 5e-3
        c1 = p[0] + st[0] * (p[1] - p[0]); c2 = p[2] + st[1] * (p[3] - p[2])
        assert np.allclose(c2 - c1, dv, atol=1e-14)


def test_point_triangle_bruteforce(built):
    rng = np.random.default_rng(3)
    g = np.linspace(0, 1, 201)
    V, W = np.meshgrid(g, g)
    m = V + W <= 1
    V, W = V[m], W[m]
    for _ in range(60):
        p = rng.standard_normal((4, 3))
        dv, vw = O.point_triangle(*p)
        q = (1 - V - W)[:, None] * p[1] + V[:, None] * p[2] + W[:, None] * p[3]
        d = np.linalg.norm(q - p[0], axis=1).min()
        assert np.linalg.norm(dv) <= d + 1e-12 and np.linalg.norm(dv) >= d - 1e-2
        cp = (1 - vw.sum()) * p[1] + vw[0] * p[2] + vw[1] * p[3]
        assert np.allclose(cp - p[0], dv, atol=1e-14)
        assert vw.min() >= 0 and vw.sum() <= 1 + 1e-15


def test_pair_compute_semantics(built):
    """dc points from element 1 to element 2 and joins the two barycentric points."""
    rng = np.random.default_rng(4)
    for _ in range(100):
        t1 = rng.standard_normal((3, 3))
        t2 = rng.standard_normal((3, 3)) + rng.standard_normal(3) * 2
        r = O.pair_compute(t1, t2)
        p1 = (1 - r["v"][0] - r["w"][0]) * t1[0] + r["v"][0] * t1[1] + r["w"][0] * t1[2]
        p2 = (1 - r["v"][1] - r["w"][1]) * t2[0] + r["v"][1] * t2[1] + r["w"][1] * t2[2]
        assert np.allclose(p2 - p1, r["dc"], atol=1e-12)
        assert abs(r["d2"] - r["dc"] @ r["dc"]) <= 1e-15 * max(r["d2"], 1)


def test_friction_state_machine(built):
    n = np.array([0.0, 0.0, 1.0])
    cp = np.array([0.1, 0.2, 0.3])
    # slow tangential motion with a normal force: a static spring is created
    # (the spring starts at the dynamic force mu_d f_n, so the transition is continuous)
    E, fc, st, so = O.friction_apply(1.0, n, np.array([1e-4, 0, 0]), 0.0, 1e-3, 10.0, 0.5, 0.3, 0.0, 0,
                                     np.zeros(3), cp)
    assert st == 1 and np.linalg.norm(so) > 0
    assert abs(fc[0] + 0.3) < 1e-6 and fc[2] == 0.0
    # continuing to stick: origin kept, spring force grows with displacement
    E2, fc2, st2, so2 = O.friction_apply(1.0, n, np.array([1e-4, 0, 0]), 0.0, 1e-3, 10.0, 0.5, 0.3, 0.0, st, so,
                                         cp + np.array([0.005, 0, 0]))
    assert st2 == 1 and np.array_equal(so2, so) and fc2[0] < fc[0] and E2 > 0
    # fast motion: dynamic friction mu_d * f_n opposite to the velocity
    E3, fc3, st3, so3 = O.friction_apply(2.0, n, np.array([1.0, 0, 0]), 0.0, 1e-3, 10.0, 0.3, 0.25, 0.0, 1, so,
                                         cp)
    assert st3 == 0 and E3 == 0 and np.allclose(fc3, [-0.5, 0, 0], rtol=1e-7) and not so3.any()
    # no normal force: never sticks
    E4, fc4, st4, _ = O.friction_apply(0.0, n, np.array([1e-5, 0, 0]), 0.0, 1e-3, 10.0, 0.3, 0.3, 0.0, 0,
                                       np.zeros(3), cp)
    assert st4 == 0 and not fc4.any()


def test_fixed_order_sum_matches_definition(built):
    rng = np.random.default_rng(5)
    x = rng.random(5000)
    lanes = np.zeros(1024)
    for l in range(1024):
        s = 0.0
        for i in range(l, len(x), 1024):
            s += x[i]
        lanes[l] = s
    st = 512
    while st > 0:
        lanes[:st] = lanes[:st] + lanes[st:2 * st]
        st //= 2
    assert O.fixed_order_sum(x) == lanes[0]


def test_contact_list_equals_bruteforce(mesh3):
    """Linked cells + filters give exactly the O(F^2) pair set at a squashed state."""
    X, T = mesh3
    from tests.common import cell_size_mult_for

    p = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
    o = O.Oracle(X, T, p, threads=2)
    rng = np.random.default_rng(6)
    u = np.zeros_like(X)
    u[:, 2] = (0.0042 - 1.0) * X[:, 2]
    u = (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)
    o.set_state(u, np.zeros_like(u), np.zeros_like(u))
    o.rebuild_contacts()
    pairs = {tuple(x) for x in o.contact_state()["pairs"]}
    info = o.cell_info()
    P = (X.reshape(-1) + u).reshape(-1, 3)[T]
    lo, hi = P.min(axis=1), P.max(axis=1)
    d_max = info["d_max"]
    brute = set()
    for e1 in range(len(T)):
        close = set(o.close_elems(e1))
        cand = np.nonzero(~((lo[e1] > hi + d_max).any(axis=1) | (lo > hi[e1] + d_max).any(axis=1)))[0]
        for e2 in cand:
            if e2 <= e1 or e2 in close:
                continue
            if O.pair_compute(P[e1], P[e2])["d2"] <= d_max * d_max:
                brute.add((e1, int(e2)))
    assert len(pairs) > 50
    assert pairs == brute


def test_oracle_step_conserves_free_flight(mesh3):
    """Without forces (zero stiffness contribution: rigid translation at
    constant velocity, no damping), Newmark keeps u + t v exact."""
    X, T = mesh3
    p = physics_params(contact=False, damping_alpha=0.0)
    o = O.Oracle(X, T, p, threads=1)
    v0 = np.tile([0.3, -0.1, 0.2], len(X))
    z = np.zeros_like(v0)
    o.set_state(z, v0, z)
    o.step(10)
    u, v, a = o.get_state()
    assert np.allclose(u, 10 * p.dt * v0, rtol=1e-12, atol=1e-18)
    assert np.allclose(v, v0, rtol=1e-12)


def test_oracle_adaptive_dt_grows_and_rejects():
    """Adaptive time stepping (ShellSystem.C:1010-1044, 1104-1117): a too-small
    dt grows by (target/err)^(1/3) until the error estimate is inside the band;
    a too-large one is rejected and retried smaller; the accepted steps' dt sum
    to the simulated time."""
    import numpy as np
    from shell_gb300 import lib as L
    from tests.common import classical_pressure, physics_params
    X, T = L.icosphere(3)
    u0 = L.gaussian_normal_imperfection(X, 1e-3, 0).reshape(-1)
    final = []
    for dt0 in (1e-6, 5e-2):
        p = physics_params(contact=False, dt=dt0, adapt_dt_every=1, rel_loc_err_min=5e-5, rel_loc_err_max=5e-4)
        o = O.Oracle(X, T, p, threads=4)
        o.apply_initial_conditions(u0, 0.0, -classical_pressure())
        rep, st = o.step(30, np.full(30, -classical_pressure()))
        assert rep.steps_done == 30 and st < 3
        assert abs(rep.sum_dt - o.get_time()[0]) <= 1e-15 * o.get_time()[0]
        final.append((o.dt(), o.rejections()))
    (dt_a, rej_a), (dt_b, rej_b) = final
    assert dt_a > 100 * 1e-6          # grew from a too-small step
    assert rej_b >= 1                 # a too-large first step was repeated
    assert 0.5 < dt_a / dt_b < 2.0    # both settle where the error estimate is inside the band
