"""GPU tests of the learned moment surrogate's pieces: the device MLP
(tcgen05 BF16 matmuls, GELU, MSE, Adam) against the CPU oracle, and the
device-regenerated parameter family against Hamiltonians assembled on the
host."""

import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

WIDE = [3, 256, 256, 256, 512]     # the surrogate's network
SMALL = [3, 64, 64, 96]


@pytest.fixture(scope='module')
def lib():
    from kwant_gb300 import _lib
    return _lib


def _data(widths, B, seed):
    rng = np.random.RandomState(seed)
    x = rng.uniform(-1, 1, size=(B, widths[0])).astype(np.float32)
    y = rng.normal(size=(B, widths[-1])).astype(np.float32)
    return x, y


@pytest.mark.parametrize('widths,B', [(SMALL, 96), (WIDE, 160), (WIDE, 32)])
def test_forward_matches_oracle(lib, widths, B):
    net = lib.Mlp(widths, max_batch=256, seed=5)
    p = net.get_params()
    assert p.size == mo.num_params(widths)
    x, _ = _data(widths, B, 1)
    got = net.forward(x)
    ref, _ = mo.forward(p, x, widths, emulate_bf16=True)
    scale = np.abs(ref).max()
    # BF16 operands identical, FP32 (device) vs FP64 accumulation, plus
    # rare one-ulp BF16 flips of hidden activations
    assert np.abs(got - ref).max() <= 2e-3 * scale
    assert np.linalg.norm(got - ref) <= 2e-4 * np.linalg.norm(ref)
    exact, _ = mo.forward(p, x, widths)
    assert np.linalg.norm(got - exact) <= 3e-2 * np.linalg.norm(exact)


@pytest.mark.parametrize('widths,B', [(SMALL, 64), (WIDE, 128)])
def test_gradients_match_oracle(lib, widths, B):
    net = lib.Mlp(widths, max_batch=256, seed=7)
    p = net.get_params()
    x, y = _data(widths, B, 2)
    g, loss = net.gradients(x, y)
    lref, gref = mo.loss_and_grads(p, x, y, widths, emulate_bf16=True)
    assert loss == pytest.approx(lref, rel=1e-4)
    assert np.linalg.norm(g - gref) <= 1e-3 * np.linalg.norm(gref)
    # per layer, weights and biases separately
    off = 0
    for k, n in zip(widths[:-1], widths[1:]):
        for size in (n * k, n):
            a, b = g[off:off + size], gref[off:off + size]
            assert np.linalg.norm(a - b) <= 3e-3 * np.linalg.norm(b), off
            off += size
    _, gexact = mo.loss_and_grads(p, x, y, widths)
    assert np.linalg.norm(g - gexact) <= 5e-2 * np.linalg.norm(gexact)


def test_adam_step_matches_oracle(lib):
    widths = SMALL
    net = lib.Mlp(widths, max_batch=64, seed=9)
    p0 = net.get_params()
    x, y = _data(widths, 64, 3)
    g, _ = net.gradients(x, y)
    net.train(x, y, batch=64, epochs=1, lr=1e-3, seed=0)
    p1 = net.get_params()
    ref, _, _ = mo.adam_step(p0, g, 0.0, 0.0, 1, 1e-3)
    # the step uses a shuffled copy of the same batch: the gradient agrees
    # to FP32 summation order, so compare where |g| is not tiny
    big = np.abs(g) > 1e-5 * np.abs(g).max() + 1e-7
    assert big.sum() > 0.5 * g.size
    assert np.abs(p1 - ref)[big].max() <= 2e-6


def test_set_params_roundtrip_and_training(lib):
    widths = [3, 64, 64, 32]
    net = lib.Mlp(widths, max_batch=128, seed=1)
    rng = np.random.RandomState(4)
    p = mo.glorot_init(widths, rng)
    net.set_params(p)
    assert np.array_equal(net.get_params(), p)
    x = rng.uniform(-1, 1, size=(512, 3)).astype(np.float32)
    n = np.arange(32)
    y = np.cos(np.outer(x[:, 0] + 0.5 * x[:, 1] * x[:, 2], n) *
               0.05).astype(np.float32)
    l0, _ = mo.loss_and_grads(p, x, y, widths)
    last = net.train(x, y, batch=64, epochs=60, lr=3e-3, seed=1)
    assert last < 0.05 * l0
    pred = net.forward(x)
    assert np.mean((pred - y) ** 2) == pytest.approx(last, rel=0.5)


def test_mlp_rejects_bad_shapes(lib):
    with pytest.raises(ValueError):
        lib.Mlp([3, 100, 32])            # hidden width not a multiple of 32
    with pytest.raises(ValueError):
        lib.Mlp([3, 64, 40])             # output width not a multiple of 32
    net = lib.Mlp([3, 64, 32], max_batch=64)
    x = np.zeros((48, 3), np.float32)
    with pytest.raises(ValueError):
        net.gradients(x, np.zeros((48, 32), np.float32))   # 48 % 32 != 0


# ------------------------------------------------------------------ family
def _moments(lib, H, a, b, prec, vecs, M, reorder=False):
    h = lib.Handle(H, a, b, prec, reorder=reorder)
    blk = lib.Block(h, vecs)
    out = blk.dos_moments(0, M)
    blk.close()
    h.close()
    return out


@pytest.mark.parametrize('prec,reorder,tol', [
    ('fp64', False, 1e-11), ('mixed', False, 2e-6), ('mixed', True, 2e-6)])
def test_family_point_matches_host_hamiltonian(lib, prec, reorder, tol):
    from kwant_gb300 import lattices
    P = {'fp64': lib.PREC_FP64, 'mixed': lib.PREC_MIXED}[prec]
    fam = lattices.honeycomb_family(30, seed=2)
    lo, hi = fam.gershgorin_bounds(((0, 0.02), (0, 3), (0, 0.3)))
    a, b = (hi - lo) / 1.95, (hi + lo) / 2
    N = fam.shape[0]
    vecs = np.exp(2j * np.pi * np.random.RandomState(3).random_sample((4, N)))
    M = 64
    h = lib.Handle(fam.hamiltonian(0.01, 1.5, 0.15), a, b, P, reorder=reorder)
    h.family_set(fam.base, fam.theta, fam.d1, fam.d2)
    blk = lib.Block(h, vecs)
    for pt in [(0.0, 0.0, 0.0), (0.019, 2.7, 0.05), (0.004, 0.3, 0.29)]:
        h.family_point(*pt)
        blk.rewind()
        got = blk.dos_moments(0, M)
        ref = _moments(lib, fam.hamiltonian(*pt), a, b, P, vecs, M, reorder)
        assert np.abs(got - ref).max() <= tol * N, pt
    blk.close()
    h.close()


def test_family_rejects_other_structure(lib):
    from kwant_gb300 import lattices
    fam = lattices.honeycomb_family(6, seed=0)
    other = lattices.honeycomb(6, 1.0, 0.0, 0.0, 0.0).hamiltonian_submatrix(
        sparse=True)     # exact zeros dropped: fewer entries
    h = lib.Handle(fam.hamiltonian(0.0, 1.0, 0.1), 5.0, 0.0, lib.PREC_MIXED)
    with pytest.raises(ValueError):
        h.family_set(other, fam.theta, fam.d1, fam.d2)
    shuffled = fam.d1.copy()
    shuffled.indices = shuffled.indices[::-1].copy()
    with pytest.raises(ValueError):
        h.family_set(fam.base, fam.theta, shuffled, fam.d2)
    with pytest.raises(ValueError):
        h.family_point(0.0, 1.0, 0.0)      # nothing set yet
    h.close()


def test_block_randomize(lib):
    from kwant_gb300 import lattices
    fam = lattices.honeycomb_family(12, seed=1)
    H = fam.hamiltonian(0.01, 1.0, 0.1)
    N = H.shape[0]
    for prec, tol in ((lib.PREC_FP64, 1e-12), (lib.PREC_MIXED, 1e-6)):
        h = lib.Handle(H, 5.0, 0.0, prec)
        blk = lib.Block(h, np.ones((5, N), complex))
        blk.randomize(7)
        m7 = blk.dos_moments(0, 16)
        # |v_i| = 1: mu_0 = N for every vector
        assert np.allclose(m7[:, 0].real, N, rtol=tol)
        blk.randomize(7)
        assert np.array_equal(blk.dos_moments(0, 16), m7)
        blk.randomize(8)
        m8 = blk.dos_moments(0, 16)
        assert np.abs(m8[:, 1:] - m7[:, 1:]).max() > 1e-3 * N
        blk.close()
        h.close()


def _truth_moments(fam, X, a, b, M):
    out = []
    for p in X:
        ev = np.linalg.eigvalsh(fam.hamiltonian(*p).toarray())
        out.append(np.cos(np.outer(np.arange(M),
                                   np.arccos((ev - b) / a))).mean(axis=1))
    return np.array(out)


def test_surrogate_beats_plain_sweep_against_exact_dos(lib):
    """What the network gains: trained on independent noisy KPM sweeps
    (R = 4 random vectors per point), its DOS is several times closer to
    the exact (diagonalisation) DOS than the plain KPM sweep's at the same
    points, at a fraction of the per-point cost."""
    from kwant_gb300 import lattices, surrogate as S
    box = ((0.0, 0.02), (0.0, 3.0), (0.0, 0.3))
    fam = lattices.honeycomb_family(16, seed=0)            # 512 sites
    M = 64
    sw = S.MomentSweep(fam, box, num_moments=M, num_vectors=4,
                       precision='mixed', rng=1, fresh_vectors=True)
    A, _ = S.dos_operator(M, sw.a, sw.b)
    Xtr = S.random_points(box, 2048, 11)
    Xte = S.random_points(box, 64, 12)
    Ytr = sw.moments(Xtr)
    Yte = sw.moments(Xte)
    truth = _truth_moments(fam, Xte, sw.a, sw.b, M)
    sur = S.MomentSurrogate(box, M, hidden=(128, 128), members=3, seed=2,
                            max_batch=1024,
                            input_map=('sqrt', 'linear', 'linear'))
    sur.fit(Xtr, Ytr, epochs=300, batch=128, lr=2e-3)
    mom, _ = sur.predict(Xte, A)
    e_kpm = np.abs((Yte - truth) @ A.T).max(axis=1)
    e_sur = np.abs((mom - truth) @ A.T).max(axis=1)
    print('DOS Linf vs exact: plain KPM median %.2e max %.2e; surrogate '
          'median %.2e max %.2e' % (np.median(e_kpm), e_kpm.max(),
                                    np.median(e_sur), e_sur.max()))
    assert np.median(e_sur) < 0.4 * np.median(e_kpm)
    assert e_sur.max() < e_kpm.max()
    sur.close()
    sw.close()


def test_surrogate_sweep_fallback_is_plain_kpm(lib):
    """Points whose estimated error exceeds tol are answered by the plain
    KPM (bit-identical to the plain sweep with the same vectors); accepted
    points stay within tol of it."""
    from kwant_gb300 import lattices, surrogate as S
    box = ((0.0, 0.02), (0.0, 3.0), (0.0, 0.3))
    fam = lattices.honeycomb_family(16, seed=0)
    M = 64
    sw = S.MomentSweep(fam, box, num_moments=M, num_vectors=4,
                       precision='mixed', rng=1)
    A, _ = S.dos_operator(M, sw.a, sw.b)
    Xtr = S.random_points(box, 1024, 11)
    Xte = S.random_points(box, 64, 12)
    Ytr = sw.moments(Xtr)
    Yte = sw.moments(Xte)
    sur = S.MomentSurrogate(box, M, hidden=(128, 128), members=3, seed=2,
                            max_batch=1024,
                            input_map=('sqrt', 'linear', 'linear'))
    sur.fit(Xtr[:-256], Ytr[:-256], epochs=300, batch=128, lr=2e-3)
    sur.calibrate(Xtr[-256:], Ytr[-256:], A)
    _, est = sur.predict(Xte, A)
    tol = float(np.median(est))
    mom, accept, info = S.SurrogateSweep(sur, sw, A, tol=tol).run(Xte)
    assert 0 < accept.sum() < len(Xte)
    assert np.array_equal(mom[~accept], Yte[~accept])
    err = np.abs((mom - Yte) @ A.T).max(axis=1)
    assert np.mean(err[accept] <= tol) >= 0.8
    sur.close()
    sw.close()


def test_ensemble_dos_on_device_matches_numpy():
    """kpm_ensemble_dos (the surrogate's DOS spread and calibration error
    on the device) against the same projections in numpy, FP64."""
    from kwant_gb300 import _lib, surrogate as S
    rng = np.random.RandomState(4)
    E, P, M = 4, 37, 96
    A, _ = S.dos_operator(M, 2.5, 0.1)
    mem = rng.randn(E, P, M) * np.exp(-np.arange(M) / 30.0)
    ref = rng.randn(P, M) * np.exp(-np.arange(M) / 30.0)
    spread, err = _lib.ensemble_dos(mem, np.ascontiguousarray(A.T), ref=ref)
    dos = mem @ A.T
    want_s = dos.std(axis=0, ddof=1).max(axis=1)
    want_e = np.abs(dos.mean(axis=0) - ref @ A.T).max(axis=1)
    assert np.allclose(spread, want_s, rtol=1e-12, atol=1e-14)
    assert np.allclose(err, want_e, rtol=1e-12, atol=1e-14)
    s2, e2 = _lib.ensemble_dos(mem[:1], np.ascontiguousarray(A.T))
    assert np.all(s2 == 0.0) and e2 is None
