"""Fused graph steps against direct launches, bit for bit.

Graph steps with a fixed dt predict the next step in the corrector and defer
the corrector's linked-cell pass into the next step's IF node; direct
launches (use_graph=0) run the unfused sequence.  On a contact-heavy state
(the sphere squashed to a double layer, so the candidate list is rebuilt
during the run) the two must give the same state, candidate list, friction
state and du_sum bit for bit, however the fused steps are split into calls
(shl_step, shl_step_enqueue / shl_step_collect) and interleaved with host
accesses that read the contact state or reset the state.
"""
import numpy as np
import pytest

from shell_gb300 import lib as L
from tests.common import cell_size_mult_for, physics_params

pytestmark = pytest.mark.gpu


def squashed(X, seed=3, s=0.0042):
    rng = np.random.default_rng(seed)
    u = np.zeros_like(X)
    u[:, 2] = (s - 1.0) * X[:, 2]
    return (u + 2e-5 * rng.standard_normal(X.shape)).reshape(-1)


def bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


def _mapped_device_pointer(host_ptr):
    """Device address of a page-locked host buffer (driver API
    cuPointerGetAttribute), or 0 when the buffer is not mapped host memory."""
    import ctypes

    cu = ctypes.CDLL("libcuda.so.1")
    CU_POINTER_ATTRIBUTE_MEMORY_TYPE, CU_POINTER_ATTRIBUTE_DEVICE_POINTER, CU_MEMORYTYPE_HOST = 2, 3, 1
    mtype, dptr = ctypes.c_uint(0), ctypes.c_uint64(0)
    if cu.cuPointerGetAttribute(ctypes.byref(mtype), CU_POINTER_ATTRIBUTE_MEMORY_TYPE, ctypes.c_void_p(host_ptr)):
        return 0
    if mtype.value != CU_MEMORYTYPE_HOST:
        return 0
    if cu.cuPointerGetAttribute(ctypes.byref(dptr), CU_POINTER_ATTRIBUTE_DEVICE_POINTER, ctypes.c_void_p(host_ptr)):
        return 0
    return dptr.value


def snapshot(g):
    u, v, a = g.get_state()
    c = g.contact_state()
    return {"u": bits(u), "v": bits(v), "a": bits(a), "pairs": c["pairs"].copy(), "stick": c["stick"].copy(),
            "origin": bits(c["origin"]), "d2": bits(c["d2"]), "du_sum": c["du_sum"]}


def assert_same(s0, s1):
    for k in s0:
        if k == "du_sum":
            assert s0[k] == s1[k], k
        else:
            assert np.array_equal(s0[k], s1[k]), k


@pytest.fixture(scope="module")
def setup(built):
    X, T = L.icosphere(3)
    p = physics_params(cell_size_mult=cell_size_mult_for(X, T, 0.01))
    u0 = squashed(X)
    return X, T, p, u0


def fresh(setup):
    X, T, p, u0 = setup
    g = L.Shell(X, T, p)
    z = np.zeros_like(u0)
    g.set_state(u0, z, z)
    g.rebuild_contacts()
    return g


def test_fused_steps_match_direct(cuda_ok, setup):
    n = 24
    table = np.zeros(n)
    d = fresh(setup)
    rd, sd = d.step(n, table, use_graph=False)
    ref = snapshot(d)
    assert rd.n_rebuilds >= 2  # the run exercises both linked-cell passes
    d.close()

    # one call of graph steps
    g = fresh(setup)
    rg, sg = g.step(n, table, use_graph=True)
    assert (rg.steps_done, rg.n_rebuilds, sg) == (rd.steps_done, rd.n_rebuilds, sd)
    assert_same(snapshot(g), ref)
    g.close()

    # split into calls, with host accesses between them
    g = fresh(setup)
    g.step(5, table[:5], use_graph=True)
    g.contact_state()                      # completes a pending pass
    u, v, a = g.get_state()
    g.set_state(u, v, a)                   # the prediction is made again
    g.upload_pressure_table(table[5:13])
    g.step_enqueue(8)                      # enqueued without collecting ...
    g.contact_state()                      # ... a host read completes the pending pass
    g.upload_pressure_table(table[13:19])
    g.step_enqueue(6)
    g.step_collect()
    g.step(3, table[19:22], use_graph=False)  # direct launches after fused ones
    g.step(2, table[22:24], use_graph=True)
    assert_same(snapshot(g), ref)
    g.close()


def test_state_through_mapped_host_memory(cuda_ok, setup):
    """shl_set_state / shl_get_state with page-locked (mapped) host buffers take the
    one-kernel path; the results equal those of pageable buffers bit for bit."""
    torch = pytest.importorskip("torch")
    X, T, p, u0 = setup
    rng = np.random.default_rng(11)
    v0 = 1e-4 * rng.standard_normal(u0.shape)
    a0 = 1e-3 * rng.standard_normal(u0.shape)
    table = np.zeros(6)
    out = []
    for pinned in (False, True):
        g = L.Shell(X, T, p)
        if pinned:
            hu, hv, ha = (torch.from_numpy(x.copy()).pin_memory().numpy() for x in (u0, v0, a0))
            # the library takes its one-kernel path only for mapped page-locked memory
            for x in (hu, hv, ha):
                assert _mapped_device_pointer(x.ctypes.data), "pinned buffer is not mapped into the device"
        else:
            hu, hv, ha = u0.copy(), v0.copy(), a0.copy()
        g.set_state(hu, hv, ha)
        g.rebuild_contacts()
        for k in range(3):
            g.step(2, table[2 * k:2 * k + 2])
            g.get_state(out=(hu, hv, ha))
            g.set_state(hu, hv, ha)
        out.append([bits(x.copy()) for x in (hu, hv, ha)])
        g.close()
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
