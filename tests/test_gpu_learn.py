"""Learned plan selection, device side: the CUDA training kernels against the
float64 oracle, and a short training run."""
import numpy as np
import pytest

from librett_gb300 import _lib
from librett_gb300.learn import train as T
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu
NF = _lib.load().librett_c_mlp_feature_count()


def test_gradients_match_float64_oracle(cuda):
    import torch

    rng = np.random.default_rng(4)
    for batch in (1, 7, 64, 300):
        params = T.init_params(NF, rng)
        params[-129:-1] = rng.normal(0, 0.3, 128)
        X = rng.normal(size=(batch, NF)).astype(np.float32)
        y = rng.normal(size=batch).astype(np.float32)
        net = T.GpuMlp(params, batch)
        loss, g = net.gradients(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda())
        ref_loss, ref_g = M.mse_gradients(params, X, y)
        assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss))
        scale = np.abs(ref_g).max()
        assert np.max(np.abs(g - ref_g)) <= 2e-4 * scale, batch
        out = net.forward(torch.from_numpy(X).cuda()).cpu().numpy()
        ref_out, _ = M.forward(params, X)
        assert np.allclose(out, ref_out, rtol=1e-4, atol=1e-4)


def test_training_reduces_loss(cuda):
    rng = np.random.default_rng(5)
    X = rng.normal(size=(4096, NF)).astype(np.float32)
    w = rng.normal(size=NF)
    y = (np.tanh(X @ w / 4.0) + 0.1 * X[:, 0] ** 2).astype(np.float32)
    params, mean, std, ym, ys, hist = T.train(X, y, epochs=20, batch=512, lr=3e-3, log=False)
    assert hist[-1] < 0.2 * hist[0]
    pred = T.predict_gpu(params, (X - mean) / std) * ys + ym
    assert np.corrcoef(pred, y)[0, 1] > 0.95
