"""The warm-start MLP: the numpy oracle's backward pass against finite differences (CPU), and
the CUDA kernels' forward pass and gradients against the oracle with the kernels' bfloat16
roundings (GPU).  Tolerances: bf16 keeps 8 significant bits, so single entries may differ by
one bf16 step where an activation rounds the other way; the whole gradient must agree to 1e-2
relative L2 error and 0.9999 cosine, the forward outputs to 2 % of their spread."""
import numpy as np
import pytest

import mlp_ref as R


def _random_model(rng, scale=1.0):
    p = rng.standard_normal(R.N_PARAM) * 0.2 * scale
    norm = np.concatenate([rng.standard_normal(R.N_IN) * 0.1, rng.uniform(0.5, 2.0, R.N_IN),
                           rng.standard_normal(R.N_OUT) * 0.1, rng.uniform(0.5, 2.0, R.N_OUT), [1.0]])
    return p.astype(np.float32), norm.astype(np.float32)


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p, norm = _random_model(rng)
    x = rng.standard_normal((12, R.N_IN))
    t = rng.standard_normal((12, R.N_OUT))
    p64 = p.astype(np.float64)
    _, g = R.loss_and_grad(p64, norm, x, t, bf16=False)
    idx = rng.choice(R.N_PARAM, 60, replace=False)
    idx = np.concatenate([idx, [R.OFF_B1, R.OFF_B2, R.OFF_B3, R.OFF_W3, R.N_PARAM - 1]])
    eps = 1e-6
    for i in idx:
        a, b = p64.copy(), p64.copy()
        a[i] += eps
        b[i] -= eps
        fd = (R.loss_and_grad(a, norm, x, t, bf16=False)[0] - R.loss_and_grad(b, norm, x, t, bf16=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0], np.float32)
    y = R.bf16(x)
    assert y[0] == 1.0 and y[5] == 0.0 and y[4] == -2.5
    assert y[1] == 1.0                     # tie, to even
    assert y[2] == np.float32(1.0 + 2 ** -6)   # tie, to even (upwards)
    assert y[3] == 1.0


@pytest.mark.gpu
def test_gpu_forward_matches_oracle(gpu_lib):
    from jbgpu.lib import Mlp
    rng = np.random.default_rng(2)
    p, norm = _random_model(rng)
    m = Mlp(seed=3)
    m.set_params(p, norm)
    x = (rng.standard_normal((1000, R.N_IN)) * 2).astype(np.float32)
    y = m.forward(x)
    ref, _ = R.forward(p, norm, x, bf16=True)
    spread = np.abs(ref).max()
    assert np.max(np.abs(y - ref)) <= 0.02 * spread, np.max(np.abs(y - ref)) / spread
    m.close()


@pytest.mark.gpu
def test_gpu_gradients_match_oracle(gpu_lib):
    from jbgpu.lib import Mlp
    rng = np.random.default_rng(4)
    p, norm = _random_model(rng)
    m = Mlp(seed=5)
    m.set_params(p, norm)
    x = rng.standard_normal((700, R.N_IN)).astype(np.float32)   # not a multiple of 64: a partial tile
    t = rng.standard_normal((700, R.N_OUT)).astype(np.float32)
    g, loss = m.gradients(x, t)
    loss_ref, g_ref = R.loss_and_grad(p, norm, x, t, bf16=True)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    assert rel < 1e-2 and cos > 0.9999, (rel, cos)
    for lo, hi in [(R.OFF_W1, R.OFF_B1), (R.OFF_W2, R.OFF_B2), (R.OFF_W3, R.OFF_B3), (R.OFF_B1, R.OFF_W2)]:
        blk = np.linalg.norm(g[lo:hi] - g_ref[lo:hi]) / np.linalg.norm(g_ref[lo:hi])
        assert blk < 2e-2, (lo, blk)
    m.close()


@pytest.mark.gpu
def test_gpu_training_fits_a_smooth_target(gpu_lib):
    from jbgpu.lib import Mlp
    rng = np.random.default_rng(6)
    n = 20000
    x = rng.standard_normal((n, R.N_IN)).astype(np.float32)
    A = rng.standard_normal((R.N_IN, R.N_OUT)) * 0.3
    t = (np.tanh(x @ A) + 0.1 * np.sin(x[:, :3])).astype(np.float32)
    m = Mlp(seed=7)
    norm = np.concatenate([np.zeros(R.N_IN), np.ones(R.N_IN), np.zeros(R.N_OUT), np.ones(R.N_OUT), [1.0]]).astype(np.float32)
    m.set_params(norm=norm)
    losses = m.train(x, t, epochs=12, batch=512, lr=3e-3, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.1 * losses[0], losses
    y = m.forward(x[:2000])
    assert np.mean((y - t[:2000]) ** 2) < 0.1 * np.mean(t[:2000] ** 2)
    m.close()
