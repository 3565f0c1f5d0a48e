"""CPU checks of the surrogate network's oracle (no GPU): backpropagation
against central finite differences in FP64, the bfloat16 rounding helper,
Adam's first step, and the host-side parameter family."""

import numpy as np
import pytest

from oracle import mlp_oracle as mo


def test_backprop_matches_finite_differences():
    widths = [3, 32, 32, 32]
    rng = np.random.RandomState(0)
    p = mo.glorot_init(widths, rng).astype(np.float64)
    p[-32:] = rng.normal(size=32) * 0.1            # non-zero output bias
    x = rng.uniform(-1, 1, size=(8, 3))
    y = rng.normal(size=(8, 32))
    _, g = mo.loss_and_grads(p, x, y, widths)
    idx = rng.choice(p.size, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp = _loss64(p + e, x, y, widths)
        lm = _loss64(p - e, x, y, widths)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1e-2, abs(fd)), (i, fd, g[i])


def _loss64(p, x, y, widths):
    h = np.asarray(x, np.float64)
    layers = []
    off = 0
    for k, n in zip(widths[:-1], widths[1:]):
        W = p[off:off + n * k].reshape(n, k)
        off += n * k
        b = p[off:off + n]
        off += n
        layers.append((W, b))
    for l, (W, b) in enumerate(layers):
        z = h @ W.T + b
        h = mo.gelu(z) if l + 1 < len(layers) else z
    return np.mean((h - y) ** 2)


def test_loss_and_grads_float64_path_is_exact_backprop():
    # loss_and_grads with float64 parameters must equal the loss of _loss64
    widths = [3, 32, 32]
    rng = np.random.RandomState(1)
    p = mo.glorot_init(widths, rng)
    x = rng.uniform(-1, 1, size=(16, 3))
    y = rng.normal(size=(16, 32))
    loss, _ = mo.loss_and_grads(p, x, y, widths)
    assert loss == pytest.approx(_loss64(p.astype(np.float64), x, y, widths),
                                 rel=1e-13)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1e-3,
                  3.0e38], np.float32)
    r = mo.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1.0);
    # 1 + 3 * 2^-9 rounds up to 1 + 2^-7
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7
    assert r[3] == -2.5
    assert abs(r[4] - 1e-3) <= 1e-3 * 2 ** -8
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_adam_first_step_is_signed_lr():
    g = np.array([1e-2, -3.0, 5e-4])
    p, m, v = mo.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1,
                           lr=1e-3)
    assert np.allclose(p, -1e-3 * np.sign(g), rtol=1e-4)


def test_training_reduces_loss_on_smooth_map():
    widths = [3, 32, 32]
    rng = np.random.RandomState(2)
    x = rng.uniform(-1, 1, size=(256, 3))
    n = np.arange(32)
    y = np.cos(np.outer(x[:, 0] + 0.5 * x[:, 1] * x[:, 2], n) * 0.05)
    p0 = mo.glorot_init(widths, rng)
    l0, _ = mo.loss_and_grads(p0, x, y, widths)
    p, last = mo.train(p0, x, y, widths, batch=32, epochs=30, lr=3e-3)
    assert last < 0.1 * l0


def test_honeycomb_family_matches_direct_builder():
    from kwant_gb300 import lattices
    fam = lattices.honeycomb_family(7, seed=4)
    for flux, W, mass in [(0.0, 0.0, 0.0), (0.017, 2.3, 0.12)]:
        H1 = fam.hamiltonian(flux, W, mass)
        sysd = lattices.honeycomb(7, 1.0, flux, W, mass, seed=4)
        H2 = sysd.hamiltonian_submatrix(sparse=True)
        assert abs(H1 - H2).max() < 1e-14
    lo, hi = fam.gershgorin_bounds(((0, 0.02), (0, 3), (0, 0.3)))
    for pt in [(0.02, 3, 0.3), (0.0, 3, 0.0), (0.01, 0, 0.3)]:
        ev = np.linalg.eigvalsh(fam.hamiltonian(*pt).toarray())
        assert lo <= ev.min() and ev.max() <= hi
