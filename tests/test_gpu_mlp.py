"""The warm-start network's tensor-core kernels against the CPU restatement (oracle/mlp_oracle.py).

Bars: forward predictions within 2e-2 of the oracle's scale (bf16 activations: a float32-vs-float64
difference can flip one rounding); gradients of every parameter tensor within 3e-2 relative
(Frobenius norm) of the oracle's on the same batch, loss within 1e-3 relative; training reduces
the loss of a learnable regression by 10x.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu

SHAPES = [(12, 128), (128,), (128, 128), (128,), (128, 128), (128,), (128, 3), (3,)]
NAMES = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"]


def _split(v):
    out, k = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(np.asarray(v[k:k + n], np.float64))
        k += n
    return out


def _model(seed=3):
    from bullet3_gb300.warmstart import WarmStartMLP
    m = WarmStartMLP(seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    p = MO.init_params(seed)
    # non-zero biases so every bias path is exercised
    parts = _split(p)
    for i in (1, 3, 5, 7):
        parts[i] = rng.normal(0, 0.1, parts[i].shape)
    p = MO.pack(parts)
    norm = MO.identity_norm()
    norm[:12] = rng.normal(0, 0.2, 12)
    norm[12:24] = rng.uniform(0.5, 2.0, 12)
    norm[24:27] = rng.normal(0, 0.5, 3)
    norm[27:30] = rng.uniform(0.5, 2.0, 3)
    m.params = p
    m.normalization = norm
    return m, p, norm, rng


def test_params_round_trip():
    m, p, norm, _ = _model()
    assert np.array_equal(m.params, p)
    assert np.array_equal(m.normalization, norm)


@pytest.mark.parametrize("n", [1, 127, 1000, 4099])
def test_forward_matches_oracle(n):
    m, p, norm, rng = _model()
    x = rng.normal(0, 1, (n, 12)).astype(np.float32)
    y = m.predict(x)
    yo, _ = MO.forward(p, norm, x)
    scale = np.abs(yo).max() + 1e-6
    # the oracle rounds the same values to BF16; only the FP32 accumulation order inside the tensor
    # cores differs, which can move an activation's BF16 rounding by one unit (measured: at most
    # 5.2e-4 of the output scale up to 4,099 rows, 1.2e-3 at 65,536)
    assert np.abs(y - yo).max() <= 2e-3 * scale, (np.abs(y - yo).max(), scale)


@pytest.mark.parametrize("n", [64, 777, 5000])
def test_gradients_match_oracle(n):
    m, p, norm, rng = _model(5)
    x = rng.normal(0, 1, (n, 12)).astype(np.float32)
    t = rng.normal(0, 1, (n, 3)).astype(np.float32)
    g, loss = m.gradients(x, t)
    go, lo = MO.gradients(p, norm, x, t)
    # (measured: loss within 3.2e-6, every parameter block's gradient within 5.7e-5, relative)
    assert abs(loss - lo) <= 2e-5 * abs(lo)
    for name, a, b in zip(NAMES, _split(g), _split(go)):
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert err <= 2e-4, (name, err)
    # parameters are untouched by a gradient evaluation
    assert np.array_equal(m.params, p)


def test_training_reduces_loss():
    from bullet3_gb300.warmstart import WarmStartMLP
    rng = np.random.Generator(np.random.PCG64(11))
    n = 32768
    x = rng.normal(0, 1, (n, 12)).astype(np.float32)
    A = rng.normal(0, 0.5, (12, 3))
    t = (np.tanh(x @ A) + 0.1 * x[:, :3] ** 2).astype(np.float32)
    m = WarmStartMLP(seed=1)
    m.fit_normalization(x, t)
    m.set_training_data(x, t)
    first = m.train(steps=1, batch=1024, lr=0.0)
    last = None
    for epoch in range(6):
        last = m.train(steps=n // 1024, batch=1024, lr=2e-3, first_batch=0)
    assert last < 0.1 * first, (first, last)
    pred = m.predict(x[:2048])
    resid = np.mean((pred - t[:2048]) ** 2) / np.var(t[:2048])
    assert resid < 0.1
