"""The contact CSR's order on the GPU at a contact-heavy state.

k_csr_fill scatters each node's contact entries with atomics, so their order
in a segment depends on the scheduling; k_csr_sort (one warp per node, up to
2048 entries) and k_csr_sort_big (one block per node above that) sort every
segment, and the gather adds the node's shares in that order.  The level-6
shell squashed to a double layer with SMOOTH contact (6.3 M pairs) has nodes
on both sides of 2048 entries.  Two contexts built from the same state must
then give the same pair list and forces bit for bit: an entry that a sort
left out of order would carry the atomics' order into the sums."""
import numpy as np
import pytest

from shell_gb300 import lib as L
from shell_gb300.workloads import squashed_state, workload

pytestmark = pytest.mark.gpu


def test_contact_order_deterministic_with_large_node_segments(cuda_ok):
    X, T, p, _ = workload(L, 6, contact=L.CONTACT_SMOOTH)
    u = squashed_state(X)
    z = np.zeros_like(u)
    out = []
    for _ in range(2):
        g = L.Shell(X, T, p)
        g.set_state(u, z, z)
        f = g.eval_forces(u, z, 0.0)[0]
        pairs = np.asarray(g.contact_state()["pairs"]).reshape(-1, 2)
        out.append((f, pairs))
        g.close()
    (f0, p0), (f1, p1) = out
    # entries per node: each pair adds one to each node of both faces
    per_node = np.bincount(T[p0].reshape(-1), minlength=len(X))
    assert per_node.max() > 2048 and np.median(per_node) <= 2048
    assert np.array_equal(p0, p1)
    assert np.array_equal(f0.view(np.uint64), f1.view(np.uint64))
