"""The learned subdivision schedule: the BF16 MLP kernels against the double-precision oracle
(oracle/mlp_ref.py), training on the GPU, and what the trained network gains over the heuristic."""
import os

import numpy as np
import pytest

from oracle import mlp_ref
from rsa_mpi_gb300 import _lib
from rsa_mpi_gb300 import schedule as S

pytestmark = pytest.mark.gpu


def _random_problem(n, seed):
    rng = np.random.default_rng(seed)
    master = S.init_weights(seed)
    master[mlp_ref.NW - 66:] += rng.normal(0, 0.1, 66).astype(np.float32)  # nonzero output biases too
    wb = S.to_bf16(master)
    X = rng.random((n, 16)).astype(np.float32)
    T = rng.random((n, 2)).astype(np.float32)
    T[rng.random((n, 2)) < 0.5] = np.nan  # one action taken per sample
    T[np.all(np.isnan(T), axis=1), 0] = 0.5
    return master, wb, X, T


def test_forward_matches_double_oracle():
    master, wb, X, _ = _random_problem(3000, 1)
    y_gpu = S.forward(wb, X)
    y_ref, _ = mlp_ref.forward(mlp_ref.bf16_to_f64(wb), X)
    np.testing.assert_allclose(y_gpu, y_ref, rtol=1e-4, atol=1e-5)


def test_gradients_match_double_oracle():
    master, wb, X, T = _random_problem(2000, 2)
    m = master.copy()
    w = wb.copy()
    loss, grad = S.train_step(m, w, X, T, 0.0)  # lr 0: gradients only
    loss_ref, grad_ref = mlp_ref.loss_and_grad(mlp_ref.bf16_to_f64(wb), X, T)
    assert loss == pytest.approx(loss_ref, rel=1e-4)
    # FP32 accumulation over 2000 samples against double: relative 1e-3 of the largest gradient
    scale = np.abs(grad_ref).max()
    np.testing.assert_allclose(grad, grad_ref, rtol=1e-3, atol=1e-4 * scale)
    np.testing.assert_array_equal(m, master)


def test_training_step_descends():
    master, wb, X, T = _random_problem(1000, 3)
    losses = [S.train_step(master, wb, X, T, 0.05)[0] for _ in range(200)]
    assert losses[-1] < 0.5 * losses[0]
    # the bf16 copy is the rounded master
    np.testing.assert_array_equal(wb, S.to_bf16(master))


@pytest.mark.skipif(not os.path.exists(S.WEIGHTS), reason="no trained weights")
def test_trained_schedule_gain_over_heuristic():
    """Held-out case (4D, r = 0.02: no 4D case is in the training set): both schedules give valid, certified
    maximal packings with the same statistics, and the trained network reaches maximality in less time than the
    heuristic: the median of 5 runs at least 3 % below the heuristic's median."""
    import statistics
    _, wb = S.load()
    case = (4, [1.0] * 4, [(0.02, 1.0, 0)])
    res = {}
    for name, sch, w in (("heuristic", _lib.RSAGPU_SCHEDULE_HEURISTIC, None), ("learned", _lib.RSAGPU_SCHEDULE_LEARNED, wb)):
        times = []
        for rep in range(5):
            out = S.run_case(*case, seed=5, schedule=sch, weights_bf16=w)
            assert out["check"] == (0, 0) and out["stats"]["maximal"] == 1
            times.append(out["stats"]["ms_total"])
        res[name] = (statistics.median(times), out["stats"]["rounds"], out["fraction"])
    print("learned vs heuristic (median ms, rounds, fraction):", res)
    assert abs(res["learned"][2] - res["heuristic"][2]) < 0.005  # same packing statistics
    assert res["learned"][0] < 0.97 * res["heuristic"][0]
