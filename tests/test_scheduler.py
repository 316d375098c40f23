"""The batch scheduler's cost model: the CUDA MLP kernels against a float64
restatement (gradients, predictions, training), and what the learned schedule
gains over FIFO on held-out cost records."""
import numpy as np
import pytest

import mlp_numpy
from gpu_inscy_gb300 import scheduler, synth


def _params(n_in, seed):
    return scheduler.CostModel(seed).init_params(n_in)


def test_numpy_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    X = rng.normal(size=(20, 5))
    y = rng.normal(size=20)
    p = _params(5, 1).astype(np.float64)
    _, g = mlp_numpy.loss_grad(p, X, y)
    for i in rng.choice(p.size, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_numpy.loss_grad(pp, X, y)[0] - mlp_numpy.loss_grad(pm, X, y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i])


def test_schedule_helpers():
    costs = [5.0, 1.0, 3.0, 3.0, 8.0]
    order = scheduler.lpt_order(costs)
    assert order[0] == 4 and sorted(order) == list(range(5))
    assert scheduler.simulate_makespan(costs, order, 2) == 11.0  # {8, 3} and {5, 3, 1}
    assert scheduler.simulate_makespan(costs, range(5), 1) == sum(costs)


def test_features_are_deterministic():
    X = synth.make_small(3)
    p = dict(synth.PARAMS["small"])
    a, b = scheduler.features(X, **p), scheduler.features(X.copy(), **p)
    assert a.shape == (len(scheduler.FEATURES),) and np.array_equal(a, b)


@pytest.mark.gpu
def test_gpu_gradient_matches_float64_restatement(engine):
    from gpu_inscy_gb300 import _lib
    rng = np.random.default_rng(1)
    for rows, n_in in ((1, 3), (37, 12), (250, 12)):
        X = rng.normal(size=(rows, n_in)).astype(np.float32)
        y = rng.normal(size=rows).astype(np.float32)
        p = _params(n_in, rows)
        loss, g = _lib.mlp_grad(p, X, y)
        want_loss, want = mlp_numpy.loss_grad(p, X, y)
        assert abs(loss - want_loss) <= 1e-4 * (1 + abs(want_loss))
        np.testing.assert_allclose(g, want, rtol=2e-3, atol=2e-5 * (1 + np.abs(want).max()))
        out = _lib.mlp_predict(p, X)
        np.testing.assert_allclose(out, mlp_numpy.forward(p, X.astype(np.float64))[0], rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_gpu_training_reduces_loss(engine):
    from gpu_inscy_gb300 import _lib
    rng = np.random.default_rng(2)
    X = rng.normal(size=(200, 6)).astype(np.float32)
    y = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2]).astype(np.float32)
    p, hist = _lib.mlp_train(_params(6, 3), X, y, 1500, 3e-3)
    assert hist.shape == (1500,)
    assert hist[-1] < 0.1 * hist[0]
    assert abs(mlp_numpy.loss_grad(p, X, y)[0] - hist[-1]) < 0.05 * hist[0]


@pytest.mark.gpu
def test_learned_schedule_beats_fifo_on_held_out_records(engine):
    recs = scheduler.load_records()
    F = np.array([r["features"] for r in recs], np.float32)
    ms = np.array([r["ms"] for r in recs])
    rng = np.random.default_rng(4)
    idx = rng.permutation(len(recs))
    test, train = idx[:len(idx) // 4], idx[len(idx) // 4:]
    model = scheduler.CostModel(seed=0).fit(F[train], ms[train])
    pred = model.predict_ms(F[test])
    err = np.abs(np.log(pred) - np.log(ms[test]))
    assert np.median(err) < 0.5  # within a factor ~1.6 for most held-out runs
    gains = []
    for s in range(20):  # random held-out batches of 24 datasets on 4 lanes
        sub = rng.choice(test, 24, replace=False)
        c = ms[sub]
        fifo = scheduler.simulate_makespan(c, range(len(sub)), 4)
        learned = scheduler.simulate_makespan(c, scheduler.lpt_order(model.predict_ms(F[sub])), 4)
        gains.append(fifo / learned)
    assert np.mean(gains) > 1.0
