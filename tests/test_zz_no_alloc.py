"""The allocation-free force entry point (shl_internal_force_noalloc).

Its callers cannot allocate device memory when they evaluate forces (for
example inside their own CUDA stream capture), so they pass device buffers
they already own and the library keeps its scratch in a static device array.
This file is collected last on purpose: if it fails, a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from shell_gb300 import lib as L
from tests.common import classical_pressure, physics_params

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _state(X, rng, amp):
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    u = np.stack([amp * x * y, amp * (z * z - 0.3), amp * np.sin(2 * x) * y], 1)
    return (u + 1e-4 * rng.standard_normal(X.shape)).reshape(-1)


@pytest.mark.parametrize("level", [3, 5])
def test_noalloc_matches_eval_forces_twice(cuda_ok, level):
    import torch

    lib = L.load()
    X, T = L.icosphere(level)
    p = physics_params(contact=False)
    g = L.Shell(X, T, p)
    rng = np.random.default_rng(100 + level)
    stream = torch.cuda.current_stream()
    f_dev = torch.empty(3 * len(X), dtype=torch.float64, device="cuda")
    for call, (amp, pres) in enumerate(((0.02, -classical_pressure()), (0.05, -3 * classical_pressure()))):
        u = _state(X, rng, amp)
        f_ref = g.eval_forces(u, np.zeros_like(u), pres)[0]
        u_dev = torch.from_numpy(u).cuda()
        f_dev.fill_(float("nan"))  # the entry point must overwrite every entry
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.shl_internal_force_noalloc(g.h, ctypes.c_void_p(u_dev.data_ptr()), pres,
                                            ctypes.c_void_p(f_dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, lib.shl_last_error()
        stream.synchronize()
        if call > 0:
            # after the first call on the device, a call takes no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        f = f_dev.cpu().numpy()
        assert np.isfinite(f).all()
        assert _rel(f, f_ref) < FORCE_TOL, (call, _rel(f, f_ref))
    g.close()


def test_noalloc_rejects_oversized_and_contact(cuda_ok):
    import torch

    lib = L.load()
    X, T = L.icosphere(6)  # 81920 faces > 32768
    g = L.Shell(X, T, physics_params(contact=False))
    u = torch.zeros(3 * len(X), dtype=torch.float64, device="cuda")
    f = torch.zeros_like(u)
    st = lib.shl_internal_force_noalloc(g.h, ctypes.c_void_p(u.data_ptr()), 0.0, ctypes.c_void_p(f.data_ptr()), None)
    assert st == L.SHL_ERR_CAPACITY
    assert b"393216 slots" in lib.shl_last_error()
    g.close()
    X, T = L.icosphere(3)
    g = L.Shell(X, T, physics_params(contact=True))
    u = torch.zeros(3 * len(X), dtype=torch.float64, device="cuda")
    f = torch.zeros_like(u)
    st = lib.shl_internal_force_noalloc(g.h, ctypes.c_void_p(u.data_ptr()), 0.0, ctypes.c_void_p(f.data_ptr()), None)
    assert st == L.SHL_ERR_ARG
    g.close()
