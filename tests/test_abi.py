"""CPU tests of the C ABI library: it loads, exports every entry point that
include/shl.h declares, and its host helpers behave (no GPU calls here)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from shell_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "shl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(shl_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(built):
    lib = L.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(L.exported_symbols())
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], stdout=subprocess.PIPE).stdout.decode()
    for n in names:
        assert re.search(r"\bT %s\b" % n, out), n


def test_version_and_status_strings(built):
    lib = L.load()
    assert b"sm_103a" in lib.shl_version()
    assert lib.shl_status_string(7) == b"ERROR: The solution is not finite"
    assert lib.shl_status_string(104) == b"device buffer capacity exceeded"


def test_params_default_match_reference_defaults(built):
    p = L.default_params()
    assert p.shell_mass_density == 1e3 and p.shell_young_modulus == 1e9 and p.thickness == 1e-3
    assert p.newmark_beta == 0.25 and p.newmark_gamma == 0.5 and p.dt == 1e-6
    assert p.cell_size_mult == 4 and p.cell_margin == 0.02 and p.neighbor_margin == 0.4
    assert p.friction_stop_velocity == 0.03 and p.static_friction_tol == 0.1
    assert p.shell_shell_contact == L.CONTACT_NONE and p.pressure_base == L.CS_LOCAL


def test_read_off_roundtrip(built, tmp_path):
    text = L.icosphere_off(2)
    f = tmp_path / "m.off"
    f.write_text(text)
    X, T = L.read_off(str(f))
    X2, T2 = L.icosphere(2)
    assert np.array_equal(X, X2) and np.array_equal(T, T2)
    assert T.shape == (320, 3) and X.shape == (162, 3)


def test_imperfection_deterministic(built):
    X, _ = L.icosphere(3)
    a = L.gaussian_normal_imperfection(X, 1e-3, 0)
    b = L.gaussian_normal_imperfection(X, 1e-3, 0)
    c = L.gaussian_normal_imperfection(X, 1e-3, 1)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    g = (a * X).sum(axis=1) / np.linalg.norm(X, axis=1) / 1e-3  # Gaussian amplitudes
    assert abs(g.mean()) < 0.15 and abs(g.std() - 1) < 0.1
    t = np.cross(a, X)
    assert np.abs(t).max() < 1e-15  # purely normal


def test_create_rejects_bad_params(built):
    """Argument checks run before any device work."""
    X, T = L.icosphere(2)
    m, keep = L.make_mesh(X, T)
    lib = L.load()
    h = ctypes.c_void_p()
    p = L.default_params()  # shear modulus 0: the reference asserts > 0
    assert lib.shl_create(ctypes.byref(m), ctypes.byref(p), ctypes.byref(h)) == L.SHL_ERR_ARG
    assert b"shear" in lib.shl_last_error()
    p = L.default_params(shell_shear_modulus=1.0, shell_shell_contact=7)
    assert lib.shl_create(ctypes.byref(m), ctypes.byref(p), ctypes.byref(h)) == L.SHL_ERR_ARG
