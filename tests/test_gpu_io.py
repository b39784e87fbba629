"""State files, VTU output and per-node measurement vectors.

State files keep the text layout of ShellSystem::save/load (ShellSystem.C:
2956-3153, written with 17 significant digits by shell.C:383-390), so a saved
state reads back bit for bit and a loaded context continues exactly as the
saved one.  The VTU writer follows ShellSystem::write_vtk (ShellSystem.C:
3156-3320, default stream precision of 6 significant digits, a line break
after every 256 values).  Per-node energy densities are compared with the CPU
oracle within 1e-12 relative after one force evaluation and 1e-9 after steps.
"""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from shell_gb300 import lib as L
import oracle as O
from tests.common import cell_size_mult_for, classical_pressure, physics_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def squashed_state(X, rng, s=0.0042):
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    u += 2e-5 * rng.standard_normal(X.shape)
    return u.reshape(-1)


@pytest.fixture(scope="module")
def mesh3(built):
    return L.icosphere(3)


def _contact_pair(X, T, seed):
    rng = np.random.default_rng(seed)
    p = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01), self_damping=0.01,
                       self_friction_damping=0.01)
    u = squashed_state(X, rng)
    v = 0.02 * rng.standard_normal(u.shape)
    a = 1e-3 * rng.standard_normal(u.shape)
    return p, u, v, a


def test_node_fields_match_oracle(cuda_ok, mesh3):
    X, T = mesh3
    p, u, v, a = _contact_pair(X, T, 3)
    g = L.Shell(X, T, p)
    o = O.Oracle(X, T, p, threads=4)
    for s in (g, o):
        s.set_state(u, v, a)
    pres = -classical_pressure()
    g.eval_forces(u, v, pres)
    o.eval_forces(u, v, pres)
    ng, no = g.node_fields(), o.node_fields()
    assert np.count_nonzero(no["eself"]) > 0 and np.count_nonzero(no["efric"]) > 0
    assert rel(ng["eself"], no["eself"]) < 1e-12
    assert rel(ng["efric"], no["efric"]) < 1e-12
    assert not np.any(ng["ecav"])
    Minv, _ = g.mass_damping()
    assert np.array_equal(ng["mass"], 1.0 / Minv[0::3])
    # after steps: kinetic energy densities too
    table = np.full(3, pres)
    for s in (g, o):
        s.set_state(u, v, a)
    g.step(3, table)
    o.step(3, table)
    ng, no = g.node_fields(), o.node_fields()
    for k in ("ekin", "eself", "efric"):
        assert np.count_nonzero(no[k]) > 0, k
        assert rel(ng[k], no[k]) < 1e-9, k


def _read_state_file(path):
    with open(path) as f:
        lines = f.read().split("\n")
    return lines


def test_state_file_roundtrip_and_resume(cuda_ok, mesh3, tmp_path):
    X, T = mesh3
    V = X.shape[0]
    p, u, v, a = _contact_pair(X, T, 5)
    g = L.Shell(X, T, p)
    g.set_state(u, v, a)
    g.set_time(0.0123, 123)
    g.eval_forces(u, v, 0.0)  # builds the list and the sticking springs at this state
    g.set_state(u, v, a)
    cs = g.contact_state()
    stick = cs["stick"].astype(bool)
    assert stick.sum() > 0
    rows = np.random.default_rng(1).standard_normal((3, 14))
    path = str(tmp_path / "state_000123.dat")
    g.save_state_file(path, 123, p.dt, 4.5, rows)

    # the text layout of ShellSystem::save
    lines = _read_state_file(path)
    assert lines[0] == "123"
    assert float(lines[1]) == p.dt and float(lines[2]) == 0.0123 and float(lines[3]) == 4.5
    node = np.array([[float(x) for x in ln.split("\t")] for ln in lines[4:4 + V]])
    assert node.shape == (V, 12)
    assert np.array_equal(node[:, [0, 3, 6]].reshape(-1), u)
    assert np.array_equal(node[:, [1, 4, 7]].reshape(-1), v)
    assert np.array_equal(node[:, [2, 5, 8]].reshape(-1), a)
    assert not np.any(node[:, 9:])
    assert int(lines[4 + V]) == 3
    got_rows = np.array([[float(x) for x in ln.split("\t")] for ln in lines[5 + V:8 + V]])
    assert np.array_equal(got_rows, rows)
    nc = int(lines[8 + V])
    assert nc == stick.sum()
    sc = [ln.split("\t") for ln in lines[9 + V:9 + V + nc]]
    assert np.array_equal(np.array([[int(s[0]), int(s[1])] for s in sc]), cs["pairs"][stick])
    assert np.array_equal(np.array([[float(x) for x in s[2:]] for s in sc]), cs["origin"][stick])

    # load into a fresh context: the state reads back bit for bit
    g2 = L.Shell(X, T, p)
    step, dt, wt, rows2 = g2.load_state_file(path)
    assert (step, dt, wt) == (123, p.dt, 4.5)
    assert np.array_equal(rows2, rows)
    for x, y in zip(g.get_state(), g2.get_state()):
        assert np.array_equal(x, y)
    assert g2.get_time() == g.get_time()
    c2 = g2.contact_state()
    keep = {tuple(q): i for i, q in enumerate(c2["pairs"])}
    for q, o in zip(cs["pairs"][stick], cs["origin"][stick]):
        i = keep[tuple(q)]
        assert c2["stick"][i] == 1 and np.array_equal(c2["origin"][i], o)
    # and both contexts continue identically
    table = np.full(12, -classical_pressure())
    g.step(12, table)
    g2.step(12, table)
    for x, y in zip(g.get_state(), g2.get_state()):
        assert np.array_equal(x, y)
    assert np.array_equal(g.contact_state()["pairs"], g2.contact_state()["pairs"])


def test_state_file_errors(cuda_ok, mesh3, tmp_path):
    X, T = mesh3
    p = physics_params(contact=False)
    g = L.Shell(X, T, p)
    with pytest.raises(L.ShlError):
        g.load_state_file(str(tmp_path / "missing.dat"))
    g.apply_initial_conditions(np.zeros(X.size), 0.0, 0.0)
    path = str(tmp_path / "s.dat")
    g.save_state_file(path, 0, p.dt)
    text = open(path).read().split("\n")
    short = str(tmp_path / "short.dat")
    with open(short, "w") as f:
        f.write("\n".join(text[:100]))
    with pytest.raises(L.ShlError):
        L.Shell(X, T, p).load_state_file(short)


def test_vtu_output(cuda_ok, mesh3, tmp_path):
    X, T = mesh3
    V, F = X.shape[0], T.shape[0]
    p, u, v, a = _contact_pair(X, T, 9)
    g = L.Shell(X, T, p)
    g.set_state(u, v, a)
    g.step(2, np.full(2, -classical_pressure()))
    path = str(tmp_path / "out.vtu")
    g.write_vtu(path)
    text = open(path).read()
    root = ET.fromstring(text)
    piece = root.find("UnstructuredGrid/Piece")
    assert piece.get("NumberOfPoints") == str(V) and piece.get("NumberOfCells") == str(F)
    names = [d.get("Name") for d in piece.find("PointData")]
    assert names == ["ux", "uy", "uz", "ecav", "efric", "ekin", "eself", "mass"]
    assert [d.get("Name") for d in piece.find("CellData")] == ["ebend", "etens", "kGauss", "kMean"]

    def arr(parent, name, dtype=float):
        for d in piece.find(parent):
            if d.get("Name") == name:
                lines = [ln for ln in d.text.split("\n") if ln.strip()]
                assert all(len(ln.split()) <= 256 for ln in lines)
                return np.array(d.text.split(), dtype=dtype)
        raise KeyError(name)

    uu, _, _ = g.get_state()
    nf, ef = g.node_fields(), g.element_fields()

    def close6(x, y):  # 6 significant digits
        return np.all(np.abs(x - y) <= 6e-6 * np.abs(y) + 1e-300)

    for c, nm in enumerate(("ux", "uy", "uz")):
        assert close6(arr("PointData", nm), uu[c::3])
    for nm in ("ecav", "efric", "ekin", "eself", "mass"):
        assert close6(arr("PointData", nm), nf[nm]), nm
    for nm in ("ebend", "etens", "kGauss", "kMean"):
        assert close6(arr("CellData", nm), ef[nm]), nm
    assert close6(arr("Points", "Points"), X.reshape(-1))
    assert np.array_equal(arr("Cells", "connectivity", np.int64), T.reshape(-1))
    assert np.array_equal(arr("Cells", "offsets", np.int64), 3 * np.arange(1, F + 1))
    assert np.all(arr("Cells", "types", np.int64) == 5)
