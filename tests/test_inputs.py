"""The oracle's own input generators (oracle.inputs) against the library's.

The CPU reference arm of the benchmark builds its mesh, parameters and
imperfection without the CUDA library; it times the same workload only if
these inputs are the library's bit for bit.  The icosphere text is also pinned
by the reference's own OFF files (sha256 in tests/golden/icosphere_off.json).
No GPU is needed: the library's helpers are host code.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import inputs as I
from shell_gb300 import lib as L
from shell_gb300.workloads import workload

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "icosphere_off.json")


@pytest.mark.parametrize("level", [3, 4])
def test_oracle_icosphere_matches_reference_off_files(level):
    gold = json.load(open(GOLDEN))[str(level)]
    text = I.icosphere_text(level).encode()
    assert hashlib.sha256(text).hexdigest() == gold["sha256"]
    assert len(text) == gold["bytes"]


@pytest.mark.parametrize("level", [0, 2, 3, 5])
def test_oracle_inputs_equal_library_inputs(built, level):
    assert I.icosphere_text(level) == L.icosphere_off(level)
    X, T = I.icosphere(level)
    Xl, Tl = L.icosphere(level)
    assert np.array_equal(X.view(np.uint64), Xl.view(np.uint64)) and np.array_equal(T, Tl)
    for amp, seed in ((1e-3, 0), (2.5e-2, (3 << 32) + 11)):
        u = I.gaussian_normal_imperfection(X, amp, seed)
        ul = L.gaussian_normal_imperfection(Xl, amp, seed)
        assert np.array_equal(u.view(np.uint64), ul.view(np.uint64))


@pytest.mark.parametrize("level", [3, 6])
def test_workload_identical_through_both_generators(built, level):
    X, T, p, u0 = workload(I, level)
    Xl, Tl, pl, u0l = workload(L, level)
    assert np.array_equal(X, Xl) and np.array_equal(T, Tl)
    assert np.array_equal(u0.view(np.uint64), u0l.view(np.uint64))
    assert p.as_dict() == pl.as_dict()
