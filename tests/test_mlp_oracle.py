"""The surrogate network's numpy oracle on CPU: its gradient equals a
finite-difference derivative of its own loss (exact float64 mode), so it can
stand as the reference for the GPU kernels' backward pass."""
import numpy as np

from oracle import mlp_ref


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 65504.0], np.float32)
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - x[3]) <= abs(x[3]) * 2 ** -8
    assert (r.view(np.uint32) & 0xFFFF == 0).all()


def test_oracle_gradient_is_the_derivative():
    rng = np.random.default_rng(3)
    n_in, h, n_out = 8, 16, 4
    sizes = [n_in * h, h, h * h, h, h * n_out, n_out]
    p = rng.normal(0, 0.4, sum(sizes))
    x = rng.random((32, n_in))
    t = rng.normal(0, 1, (32, n_out))
    g, loss = mlp_ref.gradient(p, x, t, n_in, h, n_out, exact=True)
    eps = 1e-6
    for i in rng.choice(p.size, 40, replace=False):
        q = p.copy()
        q[i] += eps
        lp = mlp_ref.gradient(q, x, t, n_in, h, n_out, exact=True)[1]
        q[i] -= 2 * eps
        lm = mlp_ref.gradient(q, x, t, n_in, h, n_out, exact=True)[1]
        assert abs((lp - lm) / (2 * eps) - g[i]) <= 1e-6 + 1e-4 * abs(g[i])
