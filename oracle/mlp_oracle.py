"""CPU oracle for the learned moment surrogate's network (numpy, FP64).

TEST INFRASTRUCTURE ONLY.  Nothing in the ``kwant_gb300`` package imports
this module; only ``tests/`` and ``bench.py`` use it, as the checker of the
device network's forward pass, gradients and optimiser step.

The surrogate has no counterpart in the reference (it learns the map from
model parameters to the Chebyshev moments that kwant.kpm.SpectralDensity
computes, kwant/kpm.py:163-252); this file restates the published methods
the device kernels implement:

* a multilayer perceptron with the exact GELU, x * Phi(x) (Hendrycks and
  Gimpel, "Gaussian Error Linear Units", 2016), after every hidden layer;
* the mean-squared-error loss and its gradient by reverse-mode
  differentiation (backpropagation);
* Adam (Kingma and Ba, "Adam: A Method for Stochastic Optimization", 2015)
  with bias correction.

Parameter layout (flat float32, as on the device): for each layer l,
W_l (widths[l+1] x widths[l], row-major) then b_l (widths[l+1]).

``emulate_bf16=True`` rounds the matmul operands to bfloat16 (round to
nearest even) exactly where the device does - inputs, weights, hidden
activations after GELU, and the output gradients of each layer - and
accumulates in FP64, so that the remaining difference to the device is its
FP32 accumulation order (plus rare one-ulp bfloat16 flips of GELU outputs).
"""

import numpy as np
from scipy.special import erf

SQRT_HALF = np.sqrt(0.5)
INV_SQRT_2PI = 1.0 / np.sqrt(2.0 * np.pi)


def bf16(x):
    """float32 -> bfloat16 (round to nearest, ties to even) -> float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = (u + np.uint32(0x7FFF) + ((u >> np.uint32(16)) & np.uint32(1))) \
        & np.uint32(0xFFFF0000)
    return r.view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z * SQRT_HALF))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z * SQRT_HALF)) + z * INV_SQRT_2PI * \
        np.exp(-0.5 * z * z)


def unflatten(params, widths):
    """Flat parameter vector -> list of (W, b) per layer (views)."""
    out, off = [], 0
    for k, n in zip(widths[:-1], widths[1:]):
        W = params[off:off + n * k].reshape(n, k)
        off += n * k
        b = params[off:off + n]
        off += n
        out.append((W, b))
    assert off == params.size
    return out


def num_params(widths):
    return sum(n * k + n for k, n in zip(widths[:-1], widths[1:]))


def glorot_init(widths, rng):
    """Glorot-uniform weights, zero biases (float32 flat vector)."""
    p = []
    for k, n in zip(widths[:-1], widths[1:]):
        lim = np.sqrt(6.0 / (k + n))
        p.append(rng.uniform(-lim, lim, size=n * k))
        p.append(np.zeros(n))
    return np.concatenate(p).astype(np.float32)


def forward(params, x, widths, emulate_bf16=False):
    """Returns (prediction, cache) for x (B x widths[0])."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    # device semantics: float32 master parameters and inputs; otherwise FP64
    dt = np.float32 if emulate_bf16 else np.float64
    layers = unflatten(np.asarray(params, dt), widths)
    h = rnd(np.asarray(x, dt))
    cache = []
    for l, (W, b) in enumerate(layers):
        Wr = rnd(W)
        z = h @ Wr.T
        if emulate_bf16:
            z = (z.astype(np.float32) + b.astype(np.float32)).astype(
                np.float64)
        else:
            z = z + b.astype(np.float64)
        cache.append((h, Wr, z))
        if l + 1 < len(layers):
            g = gelu(z)
            h = rnd(g.astype(np.float32)) if emulate_bf16 else g
    return z, cache


def loss_and_grads(params, x, y, widths, emulate_bf16=False):
    """MSE loss mean((pred - y)^2) and its gradient (flat, float64)."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    pred, cache = forward(params, x, widths, emulate_bf16)
    y = np.asarray(y, np.float64)
    B, D = pred.shape
    err = pred - y
    loss = float(np.mean(err * err))
    dh = 2.0 * err / (B * D)
    grads = []
    for l in range(len(cache) - 1, -1, -1):
        h, Wr, z = cache[l]
        dz = dh * gelu_grad(z) if l + 1 < len(cache) else dh
        if emulate_bf16:
            dz = dz.astype(np.float32).astype(np.float64)
        dzr = rnd(dz.astype(np.float32)) if emulate_bf16 else dz
        grads.append((dzr.T @ h, dz.sum(axis=0)))
        dh = dzr @ Wr
    flat = []
    for dW, db in reversed(grads):
        flat += [dW.ravel(), db]
    return loss, np.concatenate(flat)


def adam_step(params, grads, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); returns new (params, m, v)."""
    g = np.asarray(grads, np.float64)
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mhat = m / (1 - b1 ** step)
    vhat = v / (1 - b2 ** step)
    p = np.asarray(params, np.float64) - lr * mhat / (np.sqrt(vhat) + eps)
    return p, m, v


def train(params, x, y, widths, batch, epochs, lr, seed=0):
    """Mini-batch Adam in FP64 (shuffled epochs, floor(n / batch) steps
    each), for small CPU cross-checks; returns (params, last epoch loss)."""
    rng = np.random.RandomState(seed)
    p = np.asarray(params, np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    step = 0
    n = x.shape[0]
    last = 0.0
    for _ in range(epochs):
        perm = rng.permutation(n)
        losses = []
        for it in range(n // batch):
            idx = perm[it * batch:(it + 1) * batch]
            loss, g = loss_and_grads(p, x[idx], y[idx], widths)
            step += 1
            p, m, v = adam_step(p, g, m, v, step, lr)
            losses.append(loss)
        last = float(np.mean(losses))
    return p, last
