"""The cost model's CUDA kernels against a CPU FP64 implementation of the same
network (same bf16-rounded weights): predictions, loss and every gradient."""
import numpy as np
import pytest

from dedispersion_gb300.costmodel import MLP


def bf16_round(a: np.ndarray) -> np.ndarray:
    """float32 -> bf16 (round to nearest even) -> float32."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def reference(params, dims, x, t):
    """FP64 forward, MSE loss and backward with the weights rounded to bf16
    (the copy the device kernels read) and fp32 biases."""
    layers, off = [], 0
    for i, o in dims:
        W = bf16_round(params[off:off + i * o]).astype(np.float64).reshape(o, i)
        off += i * o
        b = params[off:off + o].astype(np.float64)
        off += o
        layers.append((W, b))
    acts, pres = [x.astype(np.float64)], []
    for li, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        pres.append(z)
        acts.append(np.maximum(z, 0) if li < len(layers) - 1 else z)
    pred = acts[-1][:, 0]
    n = x.shape[0]
    loss = np.mean((pred - t) ** 2)
    dy = (2.0 * (pred - t) / n)[:, None]
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        W, b = layers[li]
        if li < len(layers) - 1:
            dy = dy * (pres[li] > 0)
        grads.append((dy.T @ acts[li], dy.sum(axis=0)))
        dy = dy @ W
    flat = []
    for gW, gb in reversed(grads):
        flat += [gW.reshape(-1), gb]
    return pred, loss, np.concatenate(flat)


@pytest.mark.gpu
def test_forward_and_gradients_match_fp64(gpu):
    rng = np.random.default_rng(3)
    m = MLP(24, 128, 3, seed=11)
    x = rng.normal(size=(300, 24)).astype(np.float32)
    t = rng.normal(size=300).astype(np.float32)
    p = m.params()
    pred_ref, loss_ref, grad_ref = reference(p, m.dims(), x, t)
    pred = m.forward(x)
    np.testing.assert_allclose(pred, pred_ref, rtol=1e-4, atol=1e-4)
    grad, loss = m.gradients(x, t)
    assert abs(loss - loss_ref) <= 1e-4 * max(1.0, loss_ref)
    scale = np.abs(grad_ref).max()
    np.testing.assert_allclose(grad, grad_ref, rtol=1e-3, atol=1e-4 * scale)
    m.close()


@pytest.mark.gpu
def test_training_fits_a_smooth_function(gpu):
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, size=(1024, 8)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3] ** 2).astype(np.float32)
    m = MLP(8, 128, 3, seed=5)
    start = float(np.mean((m.forward(x) - t) ** 2))
    loss = m.train(x, t, steps=1500, lr=2e-3)
    assert loss < 0.05 * start and loss < 0.02
    # the master parameters moved and the bf16 copy follows them
    pred = m.forward(x)
    assert abs(float(np.mean((pred - t) ** 2)) - loss) < 1e-3
    m.close()
