"""The learned step-size controller: the network's CUDA gradient and inference against the FP64
numpy statement (oracle/mlp.py), training on the GPU, and the controller against plain step
doubling."""
import numpy as np
import pytest

from oracle import mlp as omlp


def _problem(n=300, seed=0):
    rng = np.random.default_rng(seed)
    w = (rng.standard_normal(omlp.NW) * 0.2).astype(np.float32)
    X = rng.standard_normal((n, 16)).astype(np.float32) * 3 + 1
    y = (np.sin(X[:, 0]) + 0.3 * X[:, 1] * X[:, 2] / 9).astype(np.float32)
    norm = np.concatenate([np.full(16, 1.0), np.full(16, 3.0), [0.1, 0.7]]).astype(np.float32)
    return w, X, y, norm


def test_oracle_gradient_matches_finite_differences():
    w, X, y, norm = _problem(40)
    w = w.astype(np.float64)
    _, g = omlp.loss_grad(w, X, y, norm)
    rng = np.random.default_rng(1)
    for k in rng.choice(omlp.NW, 25, replace=False):
        e = np.zeros_like(w)
        e[k] = 1e-6
        fd = (omlp.loss_grad(w + e, X, y, norm)[0] - omlp.loss_grad(w - e, X, y, norm)[0]) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, k


@pytest.mark.gpu
def test_device_gradient_and_inference_match_oracle(gpu_lib):
    from mpc_gb300.capi import MLP
    w, X, y, norm = _problem()
    mlp = MLP(0)
    mlp.set_normalization(norm[:16], norm[16:32], norm[32], norm[33])
    mlp.weights = w
    loss, g = mlp.loss_grad(X, y)
    l_ref, g_ref = omlp.loss_grad(w, X, y, norm)
    assert abs(loss / l_ref - 1) < 1e-5
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-5
    for block in (slice(0, 1024), slice(1024, 1088), slice(5248, 5313)):   # W1, b1, the last layer
        assert np.linalg.norm(g[block] - g_ref[block]) / np.linalg.norm(g_ref[block]) < 1e-4
    pred = mlp.predict(X)
    ref = omlp.forward(w, X, norm)
    assert np.max(np.abs(pred - ref)) < 1e-5 * max(1.0, np.max(np.abs(ref)))
    mlp.close()


@pytest.mark.gpu
def test_training_on_the_gpu_fits_a_smooth_function(gpu_lib):
    from mpc_gb300.capi import MLP
    rng = np.random.default_rng(3)
    X = rng.standard_normal((4096, 16)).astype(np.float32)
    y = (np.tanh(X[:, 0] + 0.5 * X[:, 3]) + 0.2 * X[:, 7] ** 2).astype(np.float32)
    mlp = MLP(7)
    mlp.set_normalization(np.zeros(16), np.ones(16), float(y.mean()), float(y.std()))
    w0 = mlp.weights
    l0, _ = mlp.loss_grad(X, y)
    loss = mlp.train(X, y, epochs=40, batch=128, lr=3e-3, seed=1)
    l1, _ = mlp.loss_grad(X, y)
    assert not np.array_equal(w0, mlp.weights)
    assert l1 < 0.05 * l0 and abs(loss - l1) < 0.5 * l0
    mlp.close()


@pytest.mark.gpu
def test_learned_controller_beats_plain_step_doubling(gpu_lib):
    """Train on step-doubling pairs of 16 small cells, then run a held-out cell: the learned
    controller executes fewer split steps than step doubling, with an end field as close to a
    fine fixed-step solution; its periodic checks run."""
    from mpc_gb300 import dzlearn
    train_cells = dzlearn.controller_cells(3000, 16, (32, 32, 256), passes=4, steps_per_pass=10, def_err=1e-4)
    for c in train_cells:
        c.cav = 0.1
    X, y = dzlearn.collect(train_cells, rounds=60)
    assert len(y) > 300 and np.isfinite(X).all() and np.isfinite(y).all()
    mlp, loss = dzlearn.fit(X, y, epochs=80, seed=0)
    assert loss < 0.5
    cell = dzlearn.controller_cells(1000, 1, (32, 32, 256), passes=2, steps_per_pass=10, def_err=1e-4)[0]
    cell.cav = 0.1
    rows = dzlearn.evaluate([cell], mlp, ref_steps_per_pass=400, safeties=(0.9,), check_every=8, fallback_len=4)
    r = rows[0]
    print(r)
    assert r["checks"] >= 1
    assert r["steps_learned"] < r["steps_plain"], r
    assert r["err_learned"] < max(1e-3, 1.5 * r["err_plain"]), r
