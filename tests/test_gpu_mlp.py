"""The sweep surrogate's BF16 tensor-core network (boids_mlp_*) against its
numpy oracle (oracle/mlp_ref.py): forward pass and gradients of every
parameter block, then training on a smooth target."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu

N_IN, H, N_OUT = 8, 256, 4
BLOCKS = ["W1", "b1", "W2", "b2", "W3", "b3"]


def blocks(v):
    sizes = [N_IN * H, H, H * H, H, H * N_OUT, N_OUT]
    out, o = {}, 0
    for name, s in zip(BLOCKS, sizes):
        out[name] = np.asarray(v[o:o + s], np.float64)
        o += s
    return out


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.fixture()
def net(boids_lib):
    s = boids_lib.Surrogate(N_IN, H, N_OUT, seed=11)
    yield s
    s.close()


def test_params_roundtrip(net):
    p = net.params()
    assert p.size == N_IN * H + H + H * H + H + H * N_OUT + N_OUT
    q = (p * 0.5 + 0.01).astype(np.float32)
    net.set_params(q)
    assert np.array_equal(net.params(), q)


@pytest.mark.parametrize("rows", [1, 37, 1000, 40000])
def test_forward_matches_oracle(net, rows):
    rng = np.random.default_rng(rows)
    p = net.params()
    p[N_IN * H:N_IN * H + H] = rng.normal(0, 0.1, H)  # non-zero biases
    net.set_params(p)
    x = rng.random((rows, N_IN), dtype=np.float32)
    y = net.predict(x)
    yr, _ = mlp_ref.forward(p, x, N_IN, H, N_OUT)
    assert rel(y, yr) < 2e-3
    ye, _ = mlp_ref.forward(p, x, N_IN, H, N_OUT, exact=True)
    assert rel(y, ye) < 3e-2


@pytest.mark.parametrize("rows", [16, 300])
def test_gradient_matches_oracle(net, rows):
    rng = np.random.default_rng(100 + rows)
    p = net.params()
    p[N_IN * H:N_IN * H + H] = rng.normal(0, 0.1, H)
    net.set_params(p)
    x = rng.random((rows, N_IN), dtype=np.float32)
    t = rng.normal(0, 1, (rows, N_OUT)).astype(np.float32)
    g, loss = net.gradient(x, t)
    gr, lr_ = mlp_ref.gradient(p, x, t, N_IN, H, N_OUT)
    ge, le = mlp_ref.gradient(p, x, t, N_IN, H, N_OUT, exact=True)
    assert loss == pytest.approx(lr_, rel=2e-3)
    gb, grb, geb = blocks(g), blocks(gr), blocks(ge)
    for name in BLOCKS:
        assert rel(gb[name], grb[name]) < 5e-3, name   # the kernels' own rounding points
        assert rel(gb[name], geb[name]) < 5e-2, name   # the float64 gradient


def test_training_fits_a_smooth_map(net):
    rng = np.random.default_rng(5)
    x = rng.random((4096, N_IN), dtype=np.float32)
    w = rng.normal(0, 1, (N_IN, N_OUT))
    t = np.sin(2.0 * x @ w).astype(np.float32)
    y0 = net.predict(x)
    loss0 = float(np.mean((y0 - t) ** 2))
    last = net.train(x, t, epochs=60, batch=256, lr=2e-3, seed=3)
    y1 = net.predict(x)
    loss1 = float(np.mean((y1 - t) ** 2))
    assert loss1 < 0.05 * loss0 and last < 0.05 * loss0


def test_fused_inference_agrees_with_training_forward(net):
    """Inference runs the whole network in one tensor-core kernel; the
    training pass runs it layer by layer.  Both round at the same points, so
    the loss of the fused outputs equals the training pass's loss up to FP32
    summation order (the two sum in different orders)."""
    rng = np.random.default_rng(5)
    p = net.params()
    p[N_IN * H:N_IN * H + H] = rng.normal(0, 0.1, H)
    net.set_params(p)
    x = rng.random((5000, N_IN), dtype=np.float32)
    t = rng.random((5000, N_OUT), dtype=np.float32)
    y = net.predict(x).astype(np.float64)
    _, loss = net.gradient(x, t)
    fused = float(np.mean((y - t) ** 2))
    assert abs(fused - loss) <= 1e-4 * loss, (fused, loss)
