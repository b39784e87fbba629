"""The learned warm start end to end on a small case: level-3 shells, plain
relaxation generates the training equilibria, the library's own BF16 network
is trained on them, and held-out problems relaxed from the prediction need
fewer steps to the same FP64 residual (1e-6) than from zero."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_warm_start_needs_fewer_steps(cuda_ok):
    from shell_gb300 import warmstart as WS
    r = WS.experiment(n_train=448, n_test=64, seed=1, batch_size=512, train_iters=2000, gen_tol=1e-5,
                      gen_max=15000, tol=1e-6, max_steps=15000, log=None, level=3, hidden=[256, 256],
                      train_batch=128, mixed=False, s_range=(0.15, 0.5), contact=False)
    plain, warm = r["test"]["fp64"]["plain"], r["test"]["fp64"]["warm"]
    assert r["generation"]["converged"] >= 0.6 * 448, r
    assert plain["converged"] >= 0.6 * 64, r
    assert warm["fallbacks"] <= 0.1 * 64, r
    assert warm["median_steps"] < plain["median_steps"], r
