"""SMOOTH self-contact on the CPU: the Loop limit-surface evaluation at any
point of a face (shl_limit.h / shl_subdiv.h, through the oracle) and the
oracle's closest-point search between two limit patches.

The reference's own evaluation (libMesh's FESubdivision and the missing
ConstrainedMinimizer.h) cannot run here, so these are known-answer tests:
limit positions at dyadic points equal the Loop limit of the explicitly
subdivided control net (to 1e-13), tangents and second derivatives equal
finite differences of the positions (through every child and level), the
evaluation at the quadrature point equals the element basis, the surface is
continuous across the children, and the search returns a constrained minimum
(no lower distance from other starts, zero projected gradient).
"""
import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import flipped_sphere, physics_params
from tests.test_oracle import _loop_subdivide


def smooth_params(**kw):
    return physics_params(shell_shell_contact=L.CONTACT_SMOOTH, **kw)


@pytest.fixture(scope="module")
def meshes(built):
    return {"ico3": L.icosphere(3), "flip": flipped_sphere(1)}


def irregular_faces(T, valence=None):
    val = np.bincount(T.ravel().astype(int))
    bad = val[T.astype(int)]
    if valence is None:
        return [e for e in range(len(T)) if (bad != 6)[e].any()]
    return [e for e in range(len(T)) if (bad == valence)[e].any()]


@pytest.mark.parametrize("N", [3, 4, 5, 7, 8, 12])
def test_subdivision_tables_are_affine(built, N):
    """Every child control point is an affine combination of the patch nodes."""
    tab = O.subdiv_table(N)
    assert tab.shape == (34, 3, 12, N + 6)
    assert np.abs(tab.sum(axis=3) - 1).max() < 1e-13


@pytest.mark.parametrize("name", ["ico3", "flip"])
def test_limit_at_quadrature_point_equals_element_basis(meshes, name):
    X, T = meshes[name]
    o = O.Oracle(X, T, smooth_params(), threads=1)
    for e in irregular_faces(T)[::5] + [0, 17, 400]:
        assert np.abs(o.limit_basis(e, 1 / 3, 1 / 3) - o.basis_at(e, 1 / 3, 1 / 3)).max() < 1e-14


@pytest.mark.parametrize("name,valence", [("ico3", 5), ("flip", 7)])
def test_limit_equals_loop_limit_at_dyadic_points(meshes, name, valence):
    """After K Loop steps of a random scalar field the limit at a level-K vertex
    is (1 - N chi) x + chi sum(neighbours), chi = 1 / (3 / (8 beta) + N); the
    library's limit evaluation must give it at every dyadic point of a face,
    including the points next to the irregular vertex (up to n = K + 1 levels)."""
    X, T = meshes[name]
    o = O.Oracle(X, T, smooth_params(), threads=1)
    rng = np.random.default_rng(3)
    val0 = rng.standard_normal(len(X))
    F0 = [tuple(int(x) for x in t) for t in T]
    K = 3
    Fk, vk = F0, list(val0)
    for _ in range(K):
        Fk, vk = _loop_subdivide(Fk, vk)
    nbr = [set() for _ in range(len(vk))]
    for a, b, c in Fk:
        nbr[a] |= {b, c}; nbr[b] |= {a, c}; nbr[c] |= {a, b}

    def limit(vid):
        N = len(nbr[vid]); t = 3 / 8 + 0.25 * np.cos(2 * np.pi / N); beta = (5 / 8 - t * t) / N
        chi = 1 / (3 / (8 * beta) + N)
        return (1 - N * chi) * vk[vid] + chi * sum(vk[j] for j in nbr[vid])

    def vertex_at(e, v, w):
        """the level-K vertex at face parameters (v, w) of face e (face's own node order)"""
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

    worst, tested = 0.0, 0
    for e in irregular_faces(T, valence)[:6]:
        ids = o.patch(e)
        r = list(T[e]).index(ids[0])  # the patch frame starts at the irregular vertex
        for i in range(2 ** K + 1):
            for j in range(2 ** K + 1 - i):
                if i == 0 and j == 0:
                    continue
                v, w = i / 2 ** K, j / 2 ** K
                lam = [0.0, 0.0, 0.0]
                lam[r], lam[(r + 1) % 3], lam[(r + 2) % 3] = 1 - v - w, v, w
                B = o.limit_basis(e, v, w)
                worst = max(worst, abs(B[:, 0] @ val0[ids] - limit(vertex_at(e, lam[1], lam[2]))))
                tested += 1
    assert tested > 200
    assert worst < 1e-13


@pytest.mark.parametrize("name", ["ico3", "flip"])
def test_limit_derivatives_by_finite_differences(meshes, name):
    """Tangents and second derivatives are the derivatives of the positions in
    all three children and at several subdivision levels (middle child at even
    and odd n included)."""
    X, T = meshes[name]
    o = O.Oracle(X, T, smooth_params(), threads=1)
    pts = [(0.6, 0.3), (0.1, 0.7), (0.4, 0.4), (0.15, 0.15), (0.07, 0.08), (0.03, 0.035), (0.02, 0.01),
           (0.004, 0.003), (1 / 3, 1 / 3)]
    for e in irregular_faces(T)[:8] + [3]:
        for v, w in pts:
            h = 1e-7 * (v + w)
            B = o.limit_basis(e, v, w)
            fv = (o.limit_basis(e, v + h, w) - o.limit_basis(e, v - h, w)) / (2 * h)
            fw = (o.limit_basis(e, v, w + h) - o.limit_basis(e, v, w - h)) / (2 * h)
            s1, s2 = np.abs(B[:, 1:3]).max(), np.abs(B[:, 3:]).max()
            assert np.abs(fv[:, 0] - B[:, 1]).max() < 1e-6 * s1, (e, v, w)
            assert np.abs(fw[:, 0] - B[:, 2]).max() < 1e-6 * s1, (e, v, w)
            assert np.abs(fv[:, 1] - B[:, 3]).max() < 1e-5 * s2, (e, v, w)
            assert np.abs(fw[:, 2] - B[:, 4]).max() < 1e-5 * s2, (e, v, w)
            assert np.abs(fw[:, 1] - B[:, 5]).max() < 1e-5 * s2, (e, v, w)
            assert abs(B[:, 0].sum() - 1) < 1e-13 and np.abs(B[:, 1:].sum(axis=0)).max() < 1e-9 * s2


def test_limit_continuous_across_children_and_levels(meshes):
    X, T = meshes["flip"]
    o = O.Oracle(X, T, smooth_params(), threads=1)
    for e in irregular_faces(T)[:10]:
        for v, w in [(0.5, 0.2), (0.2, 0.5), (0.3, 0.2), (0.25, 0.25), (0.125, 0.125), (0.2, 0.05)]:
            a = o.limit_basis(e, v * (1 - 1e-13), w * (1 - 1e-13))
            b = o.limit_basis(e, v * (1 + 1e-13), w * (1 + 1e-13))
            assert np.abs(a[:, :3] - b[:, :3]).max() < 1e-11 * np.abs(a[:, :3]).max()


def squashed(X, s=0.0042, seed=6):
    rng = np.random.default_rng(seed)
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    return (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)


def test_closest_points_are_constrained_minima(meshes):
    """At a squashed state every candidate pair's search converges to a point
    that satisfies the first-order (KKT) conditions of the constrained minimum:
    zero gradient along free directions, non-negative multipliers on active
    constraints.  The distance function over two curved triangles can have
    several local minima (the reference's search is local too); from starts
    spread over the triangles the search still ends at KKT points."""
    from tests.common import cell_size_mult_for
    X, T = meshes["ico3"]
    o = O.Oracle(X, T, smooth_params(cell_size_mult=cell_size_mult_for(X, T, 0.01)), threads=2)
    u = squashed(X)
    o.set_state(u, np.zeros_like(u), np.zeros_like(u))
    o.rebuild_contacts()
    pairs = o.contact_state()["pairs"]
    assert len(pairs) > 50
    rng = np.random.default_rng(0)
    irr = set(irregular_faces(T))
    sel = [k for k in range(len(pairs)) if pairs[k][0] in irr or pairs[k][1] in irr][:15] + list(range(0, len(pairs), 97))
    starts = [(1 / 3, 1 / 3, 1 / 3, 1 / 3)]
    for _ in range(3):
        a, b = rng.dirichlet([1, 1, 1], 2)
        starts.append((a[1], a[2], b[1], b[2]))
    for k, x0 in ((k, x0) for k in sel for x0 in starts):
        e1, e2 = (int(x) for x in pairs[k])
        x, d2, dc, it = o.smooth_closest(e1, e2, x0)
        assert it < 40, (e1, e2, x0)
        # projected gradient of f = |p2 - p1|^2 in the free directions
        J1, J2 = o.limit_eval(e1, x[0], x[1]), o.limit_eval(e2, x[2], x[3])
        r = J2[0] - J1[0]
        assert np.allclose(r, dc, rtol=0, atol=1e-15) and abs(r @ r - d2) <= 1e-15 * d2
        g = 2 * np.array([-r @ J1[1], -r @ J1[2], r @ J2[1], r @ J2[2]])
        scale = 2 * np.sqrt(d2) * max(np.abs(J1[1:3]).max(), np.abs(J2[1:3]).max())
        tol = 1e-6 * scale
        for t in range(2):
            v, w = x[2 * t], x[2 * t + 1]
            gv, gw = g[2 * t], g[2 * t + 1]
            if v > 1e-12 and w > 1e-12 and v + w < 1 - 1e-12:
                assert abs(gv) < tol and abs(gw) < tol, (e1, e2, t, g)
            elif v <= 1e-12 and w > 1e-12 and v + w < 1 - 1e-12:
                assert abs(gw) < tol and gv > -tol
            elif w <= 1e-12 and v > 1e-12 and v + w < 1 - 1e-12:
                assert abs(gv) < tol and gw > -tol
            elif v + w >= 1 - 1e-12 and v > 1e-12 and w > 1e-12:
                assert abs(gv - gw) < tol and gv + gw < tol


def test_smooth_contact_steps(meshes):
    """Stepping a squashed sphere with SMOOTH contact: pairs found, contacts
    active, no contact problem, the searches' coordinates persist per pair."""
    from tests.common import cell_size_mult_for
    X, T = meshes["ico3"]
    p = smooth_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
    o = O.Oracle(X, T, p, threads=2)
    u = squashed(X)
    o.set_state(u, np.zeros_like(u), np.zeros_like(u))
    o.rebuild_contacts()
    r, st = o.step(5)
    assert st == 0 and r.worst_problem == 0
    cs = o.contact_state()
    x = o.contact_coords()
    assert len(cs["pairs"]) == len(x) > 50 and r.last.Nc > 0
    assert np.all(x >= 0) and np.all(x[:, 0] + x[:, 1] <= 1) and np.all(x[:, 2] + x[:, 3] <= 1)
    assert np.any(np.abs(x - 1 / 3) > 1e-3)
