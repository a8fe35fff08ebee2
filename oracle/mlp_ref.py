"""TEST INFRASTRUCTURE ONLY: numpy restatement of the sweep surrogate's
network (boids_mlp_* of the library), for checking its GPU forward pass and
gradients.  No counterpart in the reference.

``forward``/``gradient`` follow the GPU kernels' arithmetic: operands rounded
to BF16 where the kernels round them (inputs, weights, hidden activations,
back-propagated errors), products accumulated in float64 here (FP32 on the
tensor cores), biases and bias gradients in full precision.  ``exact=True``
drops every BF16 rounding: the gradient of the network in float64.
"""
import numpy as np


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(p, n_in, h, n_out):
    sizes = [n_in * h, h, h * h, h, h * n_out, n_out]
    out, o = [], 0
    for s in sizes:
        out.append(np.asarray(p[o:o + s], np.float64))
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(n_in, h), b1, W2.reshape(h, h), b2, W3.reshape(h, n_out), b3


def _r(a, exact):
    return np.asarray(a, np.float64) if exact else bf16(a).astype(np.float64)


def forward(p, x, n_in=8, h=256, n_out=4, exact=False):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, h, n_out)
    x = _r(x, exact)
    W1, W2, W3 = _r(W1, exact), _r(W2, exact), _r(W3, exact)
    pre1 = x @ W1 + b1
    h1 = _r(np.maximum(pre1, 0), exact)
    pre2 = h1 @ W2 + b2
    h2 = _r(np.maximum(pre2, 0), exact)
    y = h2 @ W3 + b3
    return y, (x, W1, W2, W3, pre1, h1, pre2, h2)


def gradient(p, x, t, n_in=8, h=256, n_out=4, exact=False):
    """Mean squared error and its gradient, in the parameter layout."""
    y, (x, W1, W2, W3, pre1, h1, pre2, h2) = forward(p, x, n_in, h, n_out, exact)
    n = y.size
    dy = 2.0 * (y - np.asarray(t, np.float64)) / n
    loss = float(np.sum((y - t) ** 2) / n)
    dy16 = _r(dy, exact)
    gW3 = h2.T @ dy16
    gb3 = dy.sum(0)
    d2 = (dy16 @ W3.T) * (pre2 > 0)
    d2_16 = _r(d2, exact)
    gW2 = h1.T @ d2_16
    gb2 = d2.sum(0)
    d1 = (d2_16 @ W2.T) * (pre1 > 0)
    d1_16 = _r(d1, exact)
    gW1 = x.T @ d1_16
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return g, loss
