"""The learned branching scorer's arithmetic: the CPU restatement's gradient
against finite differences (CPU), the GPU training kernels' gradient against
the restatement, training on the GPU, and the tensor-core BF16 inference
against the restatement with BF16 rounding emulated (GPU)."""
import numpy as np
import pytest

from oracle import mlp_ref as R


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.0, 1.5, size=(n, R.N_IN)).astype(np.float32)
    y = (rng.uniform(size=n) < 0.3).astype(np.float32)
    w = rng.uniform(0.5, 2.0, size=n).astype(np.float32)
    return X, y, w


def test_restatement_gradient_matches_finite_differences():
    p = R.init_params(3).astype(np.float64)
    p += np.random.default_rng(4).normal(0, 0.05, size=p.size)  # nonzero biases
    X, y, w = _batch(40, 5)
    _, g = R.loss_grad(p, X, y, w)
    rng = np.random.default_rng(6)
    idx = np.concatenate([rng.choice(R.NPARAM, 60, replace=False), [R.NPARAM - 1]])
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (R.loss_grad(pp, X, y, w)[0] - R.loss_grad(pm, X, y, w)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_model_file_round_trip(tmp_path):
    from scs_gb300.engine import load_model_file, save_model
    p = R.init_params(1)
    path = str(tmp_path / "m.mlp")
    save_model(path, p)
    assert np.array_equal(load_model_file(path), p)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0], dtype=np.float32)
    got = R.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -6
    assert got[3] == -2.5 and got[4] == 0.0


@pytest.mark.gpu
def test_gpu_gradient_matches_restatement():
    """scs_mlp_grad (FP32 GPU kernels) against the float64 restatement:
    loss within 1e-5 relative, every gradient entry within 2e-3 relative or
    1e-5 of the largest entry."""
    from scs_gb300.engine import mlp_grad
    p = R.init_params(7)
    p += np.random.default_rng(8).normal(0, 0.05, size=p.size).astype(np.float32)
    for n, seed in ((300, 9), (4096, 10), (17, 11)):
        X, y, w = _batch(n, seed)
        loss_g, g_g = mlp_grad(p, X, y, w)
        loss_c, g_c = R.loss_grad(p, X, y, w)
        assert abs(loss_g - loss_c) <= 1e-5 * abs(loss_c)
        scale = np.abs(g_c).max()
        np.testing.assert_allclose(g_g, g_c, rtol=2e-3, atol=1e-5 * scale)


@pytest.mark.gpu
def test_gpu_training_fits_a_separable_rule():
    """Training with the engine's kernels drives the loss down on labels a
    network can express (y = [x0 + x3 > x5])."""
    from scs_gb300.engine import mlp_train
    rng = np.random.default_rng(12)
    X = rng.uniform(0, 1, size=(20000, R.N_IN)).astype(np.float32)
    y = (X[:, 0] + X[:, 3] > X[:, 5] + 0.5).astype(np.float32)
    p, losses = mlp_train(X, y, R.init_params(13), epochs=8, batch=1024, lr=3e-3, seed=1)
    assert losses[-1] < 0.5 * losses[0], losses
    acc = ((R.forward(p, X) > 0) == (y > 0.5)).mean()
    assert acc > 0.95, acc


@pytest.mark.gpu
def test_tensor_core_inference_matches_bf16_restatement():
    """scs_mlp_infer (mma.sync m16n8k16, BF16 operands, FP32 accumulate)
    against the restatement with BF16 rounding of inputs, weights and hidden
    activations: |dz| <= 1e-2 (1 + |z|), on row counts that are and are not
    multiples of the 16-row tile.  The float32 network stays within 5e-2
    (1 + |z|) of it."""
    from scs_gb300.engine import mlp_infer
    p = R.init_params(14)
    p += np.random.default_rng(15).normal(0, 0.05, size=p.size).astype(np.float32)
    for n in (16, 1000, 37):
        X, _, _ = _batch(n, 16 + n)
        z = mlp_infer(p, X)
        zb = R.forward_bf16(p, X)
        np.testing.assert_array_less(np.abs(z - zb), 1e-2 * (1 + np.abs(zb)))
        zf = R.forward(p, X)
        np.testing.assert_array_less(np.abs(z - zf), 5e-2 * (1 + np.abs(zf)))
