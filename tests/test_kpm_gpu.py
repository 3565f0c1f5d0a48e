"""GPU parity of the KPM path against the reference's golden outputs.

Every case reproduces a reference run (tests/golden/make_golden.py) with the
same Hamiltonian, the same random-vector stream (rng seed) and the same raw
spectral bounds, and compares per-vector moments, densities and energies.

Tolerances (relative to the largest magnitude of the reference quantity):
  precision='fp64'  : 1e-12 (the reference's own TOL, kwant/tests/test_kpm.py:38)
  precision='mixed' : densities / N within 1e-5 (DOS L-infinity target)
"""

import numpy as np
import pytest

from golden_io import load, csr, ref_vectors
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope='module')
def kpm():
    from kwant_gb300 import _lib, kpm
    if _lib.device_count() == 0:
        pytest.fail('no CUDA device: the GPU tests need a GB300')
    return kpm


def _sd(kpm, ham, g, **kw):
    kw.setdefault('rng', int(g['seed']))
    return kpm.SpectralDensity(ham, bounds=(g['lmin'], g['lmax']), **kw)


# --------------------------------------------------------------- DOS, fp64
def test_rmt_dos_fp64(kpm):
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5)
    assert sd._a == g['a'] and sd._b == g['b']
    assert np.array_equal(sd.energies, g['energies'])
    assert _rel(np.array(sd._moments_list), g['moments_list']) < TOL
    assert _rel(sd.densities, g['densities']) < TOL
    assert _rel(sd._gammas, g['gammas']) < TOL


def test_rmt_add_moments_bit_identical(kpm):
    """kwant/tests/test_kpm.py:481-505: add_moments == fresh run, bit for
    bit, including odd counts."""
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5)
    sd.add_moments(200)
    fresh = _sd(kpm, g['ham'], g, num_moments=400, num_vectors=5)
    assert np.array_equal(np.array(sd._moments_list),
                          np.array(fresh._moments_list))
    assert _rel(np.array(sd._moments_list), g['add_moments_list']) < TOL
    odd = _sd(kpm, g['ham'], g, num_moments=201, num_vectors=5)
    assert _rel(np.array(odd._moments_list), g['odd_moments_list']) < TOL
    even = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5)
    even.add_moments(1)
    assert np.array_equal(np.array(even._moments_list),
                          np.array(odd._moments_list))


def test_rmt_add_vectors_bit_identical(kpm):
    """kwant/tests/test_kpm.py:526-535."""
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5)
    sd.add_vectors(3)
    fresh = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=8)
    assert np.array_equal(sd.densities, fresh.densities)
    assert _rel(np.array(sd._moments_list), g['vec_moments_list']) < TOL


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_one_shot_dos_c_abi_matches_oracle(kpm, precision):
    """kpm_dos, the one-shot C entry point (handle with the RCM order in
    mixed precision, vector upload overlapped with the handle set-up,
    recursion, device reconstruction, download), against the oracle's whole
    SpectralDensity pipeline on the same vectors and bounds."""
    from kwant_gb300 import _lib
    g = load('square100')
    ham = csr(g)
    n = ham.shape[0]
    R, M = 6, 60
    _, vecs = ref_vectors(g['seed'], n, R)
    ref = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], M)
    a, b = ref['a'], ref['b']
    prec = _lib.PREC_MIXED if precision == 'mixed' else _lib.PREC_FP64
    for _ in range(2):      # a second call runs on a fresh handle
        mom, gam, rho = _lib.dos(ham, a, b, prec, vecs, M)
        tol = 1e-12 if precision == 'fp64' else 1e-5
        assert _rel(mom, ref['moments_list']) < tol
        assert _rel(rho.real, ref['densities']) < tol
        assert _rel(gam.real, ref['gammas']) < tol


def test_mixed_add_vectors_bit_identical_across_group_sizes(kpm):
    """Mixed precision: 10 vectors (a 16-vector block) plus 30 more (a
    32-vector block) give the same moments, bit for bit, as 40 vectors at
    once (two 32-vector groups): every vector sees the same row partition,
    slot and flush points whatever its block's group size."""
    g = load('square100')
    ham = csr(g)
    sd = _sd(kpm, ham, g, num_moments=40, num_vectors=10, precision='mixed')
    sd.add_vectors(30)
    fresh = _sd(kpm, ham, g, num_moments=40, num_vectors=40,
                precision='mixed')
    assert np.array_equal(np.array(sd._moments_list),
                          np.array(fresh._moments_list))
    assert np.array_equal(sd.densities, fresh.densities)


def test_rmt_operator_identity_matrix(kpm):
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5,
             operator=np.identity(20))
    assert _rel(np.array(sd._moments_list), g['op_moments_list']) < TOL
    assert _rel(sd.densities, g['op_densities']) < TOL


def test_rmt_lorentz_mean_false(kpm):
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=64, num_vectors=3,
             kernel=kpm.lorentz_kernel, mean=False)
    assert _rel(sd.densities, g['lor_densities']) < TOL


def test_rmt_call_and_integrate(kpm):
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5)
    assert _rel(sd(g['call_energies']), g['call_values']) < TOL
    assert abs(sd.integrate() - g['integrate']) < 1e-10
    f = sd.integrate(lambda e: kpm.fermi_distribution(e, 0.1, 0.05))
    assert abs(f - g['integrate_fermi']) < 1e-10
    # the batched device sweep: the same sums for a grid of (mu, T)
    grid = sd.integrate_sweep(mu=[[0.1], [-0.3]], temperature=[0.05, 0.0])
    assert grid.shape == (2, 2)
    assert abs(grid[0, 0] - g['integrate_fermi']) < 1e-10
    for i, m in enumerate((0.1, -0.3)):
        for j, T in enumerate((0.05, 0.0)):
            ref = sd.integrate(lambda e: kpm.fermi_distribution(e, m, T))
            assert abs(grid[i, j] - ref) < 1e-13 * max(1.0, abs(ref))
    with pytest.raises(ValueError):
        sd.integrate_sweep(0.0, -1.0)


def test_custom_kernel_runs_on_host_values(kpm):
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5,
             kernel=lambda m: kpm.jackson_kernel(m))
    assert _rel(sd.densities, g['densities']) < TOL


# ------------------------------------------------------ plain-KPM workload
def test_square100_fp64(kpm):
    g = load('square100')
    sd = _sd(kpm, csr(g), g, num_moments=100, num_vectors=10)
    assert _rel(np.array(sd._moments_list), g['moments_list']) < TOL
    assert _rel(sd.densities, g['densities']) < TOL


@pytest.mark.parametrize('precision', ['mixed', 'single'])
def test_square100_mixed_dos_error(kpm, precision):
    g = load('square100')
    ham = csr(g)
    n = ham.shape[0]
    sd = _sd(kpm, ham, g, num_moments=100, num_vectors=10,
             precision=precision)
    err = np.max(np.abs(sd.densities - g['densities'])) / n
    assert err < 1e-5, err


def test_mixed_dos_all_nodes_long_expansion(kpm):
    """Mixed precision against the oracle on a long expansion: graphene
    flake of 200 x 200 cells (8e4 orbitals) with a Peierls flux of 1/1000
    per hexagon and W = 0.5, R = 4, M = 2000, the same vectors and raw
    bounds.  The per-orbital DOS must be within 1e-5 at every one of the
    2M Chebyshev nodes, the outermost ones (x = +-0.99999992, where the
    reconstruction divides by sqrt(1 - x^2) ~ 4e-4) included; the plain
    complex64 recursion misses that there by an order of magnitude."""
    from kwant_gb300 import lattices
    syst = lattices.honeycomb(200, t=1.0, flux=1.0 / 1000, W=0.5, seed=0)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    n, R, M = ham.shape[0], 4, 2000
    v0, vecs = ref_vectors(1, n, R)
    lmin, lmax = ko.spectral_bounds(ham, 0.05, v0)
    ref = ko.spectral_density(ham, vecs, lmin, lmax, M)
    sd = kpm.SpectralDensity(ham, bounds=(lmin, lmax),
                             vector_factory=list(vecs), num_vectors=R,
                             num_moments=M, precision='mixed')
    assert np.array_equal(sd.energies, ref['energies'])
    err = np.abs(sd.densities.real - ref['densities'].real) / n
    assert err.max() < 1e-5, (err.max(), sd.energies[np.argmax(err)])


@pytest.mark.parametrize('model', ['rashba', 'wilson_dirac'])
def test_mixed_dos_wide_rows(kpm, model):
    """The compensated step on wider ELL rows, which it computes in
    chunks of four entries: the two-orbital Rashba square (width 12, three
    chunks) and the four-orbital Wilson-Dirac cube (13 entries, width 16,
    four chunks) against the oracle at every node of an M = 400 expansion,
    and add_vectors across a 16-vector and a 32-vector group bit-identical
    to one run."""
    from kwant_gb300 import lattices
    if model == 'rashba':
        syst = lattices.rashba_square(40, seed=2)
    else:
        syst = lattices.wilson_dirac_cubic(8, m=1.5, W=1.0, seed=2)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    n, R, M = ham.shape[0], 6, 400
    v0, vecs = ref_vectors(3, n, R)
    lmin, lmax = ko.spectral_bounds(ham, 0.05, v0)
    ref = ko.spectral_density(ham, vecs, lmin, lmax, M)
    sd = kpm.SpectralDensity(ham, bounds=(lmin, lmax),
                             vector_factory=list(vecs), num_vectors=R,
                             num_moments=M, precision='mixed')
    err = np.abs(sd.densities.real - ref['densities'].real) / n
    assert err.max() < 1e-5, err.max()
    small = kpm.SpectralDensity(ham, bounds=(lmin, lmax), rng=5,
                                num_vectors=10, num_moments=60,
                                precision='mixed')
    small.add_vectors(30)
    fresh = kpm.SpectralDensity(ham, bounds=(lmin, lmax), rng=5,
                                num_vectors=40, num_moments=60,
                                precision='mixed')
    assert np.array_equal(np.array(small._moments_list),
                          np.array(fresh._moments_list))


# --------------------------------------------------------------- operators
def test_ldos_density_where(kpm):
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Density
    g = load('honeycomb_ldos')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 1, 0), (n, 0, n)], np.zeros((n, 2)))
    dens = Density(syst, where=list(g['where']))
    sd = _sd(kpm, ham, g, operator=dens, num_moments=60, num_vectors=4)
    assert _rel(np.array(sd._moments_list), g['moments_list']) < TOL
    assert _rel(sd.densities, g['densities']) < TOL
    dsum = Density(syst, where=list(g['where']), sum=True)
    sd = _sd(kpm, ham, g, operator=dsum, num_moments=60, num_vectors=4)
    assert _rel(sd.densities, g['sum_densities']) < TOL
    dos = _sd(kpm, ham, g, num_moments=60, num_vectors=4)
    assert _rel(dos.densities, g['dos_densities']) < TOL


def test_current_chain(kpm):
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Current
    g = load('chain_current')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 1, 0), (n, 0, n)],
                         np.arange(n, dtype=float)[:, None])
    cur = Current(syst, where=[tuple(w) for w in g['where']])
    sd = _sd(kpm, ham, g, operator=cur, num_moments=200, num_vectors=5)
    assert _rel(np.array(sd._moments_list), g['moments_list']) < TOL
    assert _rel(sd.densities, g['densities']) < TOL


def test_two_orbital_operators(kpm):
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Density, Current
    g = load('rashba_ops')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 2, 0), (n // 2, 0, n)], g['positions'])
    sz = np.diag([1.0, -1.0])
    d_sum = Density(syst, onsite=sz, sum=True)
    d_loc = Density(syst, onsite=sz, where=list(g['where_sites']))
    cur = Current(syst, onsite=sz, where=[tuple(w) for w in g['hop_where']])
    kw = dict(num_moments=40, num_vectors=3)
    for op, pre in ((d_sum, 'sz_'), (d_loc, 'loc_'), (cur, 'cur_')):
        sd = _sd(kpm, ham, g, operator=op, **kw)
        assert _rel(np.array(sd._moments_list), g[pre + 'moments_list']) \
            < TOL, pre
        assert _rel(sd.densities, g[pre + 'densities']) < TOL, pre
    # MAT_ELS and ACT on the device
    assert _rel(d_loc(g['bra'], g['ket']), g['dens_loc_call']) < TOL
    assert abs(d_sum(g['bra'], g['ket']) - g['dens_sz_call']) < 1e-10
    assert abs(d_sum(g['bra']) - g['dens_sz_self']) < 1e-10
    assert _rel(cur(g['bra'], g['ket']), g['cur_call']) < TOL
    assert _rel(d_loc.act(g['ket']), g['dens_loc_act']) < TOL
    assert _rel(cur.act(g['ket']), g['cur_act']) < TOL


def test_source_operator(kpm):
    """kwant.operator.Source (kwant/operator.pyx:1003-1126) lowered to a
    density with per-site matrices i (H_aa^dagger M - M H_aa)."""
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Source
    g = load('source_ops')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 2, 0), (n // 2, 0, n)], np.zeros((n // 2, 2)))
    sx = np.array([[0, 1], [1, 0]], complex)
    s_loc = Source(syst, onsite=sx, where=list(g['where_sites']))
    s_sum = Source(syst, onsite=sx, sum=True)
    kw = dict(num_moments=30, num_vectors=3)
    for op, pre in ((s_loc, 'loc_'), (s_sum, 'sum_')):
        sd = _sd(kpm, ham, g, operator=op, **kw)
        assert _rel(np.array(sd._moments_list), g[pre + 'moments_list']) \
            < TOL, pre
        assert _rel(sd.densities, g[pre + 'densities']) < TOL, pre
    assert _rel(s_loc(g['bra'], g['ket']), g['loc_call']) < TOL
    assert abs(s_sum(g['bra'], g['ket']) - g['sum_call']) < 1e-10
    assert abs(s_sum(g['bra']) - g['sum_self']) < 1e-10
    assert _rel(s_loc.act(g['ket']), g['loc_act']) < TOL
    assert _rel(s_sum.act(g['ket']), g['sum_act']) < TOL


def test_mixed_operator_moments(kpm):
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Density
    g = load('honeycomb_ldos')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 1, 0), (n, 0, n)], np.zeros((n, 2)))
    dens = Density(syst, where=list(g['where']))
    sd = _sd(kpm, ham, g, operator=dens, num_moments=60, num_vectors=4,
             precision='mixed')
    err = np.max(np.abs(sd.densities - g['densities']))
    assert err < 1e-5 * max(1.0, np.max(np.abs(g['densities']))), err


# ------------------------------------------------------------------ bounds
def test_divergence_warning_on_tight_bounds(kpm):
    """Failure detection without a GPU fault: bounds that cut the spectrum
    make the recursion grow; the host flags it from the moments."""
    from kwant_gb300 import _lib
    g = load('rmt20')
    with pytest.warns(RuntimeWarning, match='do not enclose'):
        kpm.SpectralDensity(g['ham'], bounds=(0.5 * g['lmin'],
                                              0.5 * g['lmax']),
                            num_moments=200, num_vectors=2, rng=1)
    # the C ABI reports it as KPM_EDIVERGED, with the moments written
    _, vecs = ref_vectors(g['seed'], 20, 2)
    tight = kpm._rescale_ab(0.5 * g['lmin'], 0.5 * g['lmax'], 0.05)
    good = kpm._rescale_ab(g['lmin'], g['lmax'], 0.05)
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        h = _lib.Handle(g['ham'], *tight, prec)
        blk = _lib.Block(h, vecs, keep_a0=True)
        with pytest.raises(_lib.KPMDiverged, match='do not enclose'):
            blk.dos_moments(0, 200)
        blk.rewind()
        mom = blk.dos_moments(0, 200, diverged='return')
        big = np.abs(mom)          # grows until it overflows (complex64)
        assert blk.diverged
        assert not np.all(np.isfinite(big)) or \
            np.nanmax(big) > 10 * big[:, 0].max()
        blk.close()
        h.close()
        h = _lib.Handle(g['ham'], *good, prec)
        blk = _lib.Block(h, vecs, keep_a0=True)
        blk.dos_moments(0, 200)            # enclosing bounds: no error
        blk.close()
        h.close()
    with pytest.raises(_lib.KPMDiverged, match='kpm_dos'):
        _lib.dos(g['ham'], *tight, _lib.PREC_FP64, vecs, 200)



def test_lanczos_bounds_enclose_spectrum(kpm):
    g = load('rmt20')
    ev = np.linalg.eigvalsh(g['ham'])
    lo, hi = kpm.spectral_bounds(g['ham'], 0.05, method='lanczos')
    assert lo <= ev[0] + 1e-9 and hi >= ev[-1] - 1e-9
    assert abs(lo - ev[0]) < 0.025 * abs(ev[0]) + 1e-6
    g = load('square100')
    ham = csr(g)
    lo, hi = kpm.spectral_bounds(ham, 0.05, method='lanczos')
    # reference ARPACK bounds (tol = eps/2) agree to that tolerance
    assert abs(lo - g['lmin']) < 0.025 * abs(g['lmin'])
    assert abs(hi - g['lmax']) < 0.025 * abs(g['lmax'])


def test_default_bounds_path(kpm):
    """bounds=None: device bounds; densities match the reference within
    the effect of the bound tolerance."""
    g = load('square100')
    ham = csr(g)
    sd = kpm.SpectralDensity(ham, rng=1, num_moments=100, num_vectors=10)
    assert abs(sd._a - g['a']) < 0.03 * g['a']
    ev_max = np.max(np.abs(sd.densities))
    assert ev_max > 0


def test_arpack_bounds_reproduce_reference(kpm):
    g = load('square100')
    ham = csr(g)
    sd = kpm.SpectralDensity(ham, rng=1, num_moments=100, num_vectors=10,
                             bounds_method='arpack')
    # ARPACK itself runs on the host CPU of the test machine; its floating
    # point may differ from the machine that made the fixture.
    assert abs(sd._a - g['a']) < 1e-8 * g['a']
    assert abs(sd._b - g['b']) < 1e-8
    assert _rel(sd.densities, g['densities']) < 1e-6


# ----------------------------------------------------------- reconstruction
def test_device_dct_matches_scipy(kpm):
    from kwant_gb300 import _lib
    rs = np.random.RandomState(0)
    for M, W in ((7, 1), (64, 3), (500, 2)):
        mom = rs.randn(1, M, W) + 1j * rs.randn(1, M, W)
        nodes = ko.chebyshev_nodes(2 * M)
        gam, rho = _lib.reconstruct(mom, True, False, 1.0, _lib.KERNEL_NONE,
                                    4.0, nodes)
        ref_rho, ref_gam = ko.calc_fft_moments(mom[0])
        assert _rel(gam, ref_gam) < 1e-12
        assert _rel(rho, ref_rho) < 1e-12


def test_kernel_weights_on_device(kpm):
    from kwant_gb300 import _lib
    for M in (2, 10, 1000):
        g = _lib.kernel_weights(M, _lib.KERNEL_JACKSON)
        assert _rel(g, ko.jackson_kernel(np.ones(M))) < 1e-13
        g = _lib.kernel_weights(M, _lib.KERNEL_LORENTZ, 4.0)
        assert _rel(g, ko.lorentz_kernel(np.ones(M))) < 1e-13


# ------------------------------------------------------------ conductivity
def test_conductivity_fp64(kpm):
    g = load('conductivity')
    ham = csr(g)
    pos = g['orb_positions']
    kw = dict(rng=0, num_moments=48, num_vectors=4,
              bounds=(g['lmin'], g['lmax']))
    cond = kpm.conductivity(ham, alpha='x', beta='y', positions=pos, **kw)
    assert cond._a == g['a'] and cond._b == g['b']
    assert _rel(cond.moments_matrix, g['mu_xy']) < 1e-11
    assert _rel(cond._integral_factor, g['factor_xy']) < 1e-10
    vals = np.array([[cond(mu=m, temperature=T) for m in g['mus']]
                     for T in g['temps']])
    assert _rel(vals, g['values_xy']) < 1e-9
    cxx = kpm.conductivity(ham, alpha='x', beta='x', positions=pos, **kw)
    vals = np.array([[cxx(mu=m, temperature=T) for m in g['mus']]
                     for T in g['temps']])
    assert _rel(vals, g['values_xx']) < 1e-9
    # the vectorised (mu, temperature) sweep equals point-by-point calls
    grid = cxx.sweep(mu=np.asarray(g['mus'])[None, :],
                     temperature=np.asarray(g['temps'])[:, None])
    assert grid.shape == vals.shape
    assert _rel(grid, vals) < 1e-12
    cond.add_moments(16)
    vals = np.array([cond(mu=m, temperature=0.1) for m in g['mus']])
    assert _rel(vals, g['values_add']) < 1e-9


def _sigma_error_bound(dmu, a, b, M, mus, temps):
    """Bound on |sigma(mu + dmu) - sigma(mu)| over a (mu, T) grid.  sigma is
    linear in the moments matrix (kwant/kpm.py:720-760, :608-630):
    sigma = pref * sum_k w_k f_k / (1 - e_k^2)^2 * sum_mn mu~_mn G_nm(e_k)
    with mu~ = g g^T o mu (g[0] halved), Simpson weights w_k and
    pref = 2 * 4^2 / (2a)^2, so
    |d sigma| <= pref * sum_k |w_k| f_k / (1 - e_k^2)^2 *
                 sum_mn |g_m g_n dmu_mn| |G_nm(e_k)|."""
    from kwant_gb300.kpm import _simpson_weights
    g = ko.jackson_kernel(np.ones(M))
    g[0] /= 2
    x = ko.chebyshev_nodes(2 * M)
    m = np.arange(M)
    A = np.abs(np.outer(g, g) * dmu)
    per_node = np.empty(x.size)
    for k, e in enumerate(x):
        ex = np.exp(1j * np.arccos(e) * m)
        ep = (e - 1j * np.sqrt(1 - e * e) * m) * ex
        big = ep[None, :] * ex.real[:, None]
        big = big + big.conj().T
        per_node[k] = np.sum(A * np.abs(big.T))
    w = np.abs(_simpson_weights(x)) / (1 - x ** 2) ** 2 * per_node
    pref = 2 * 4 ** 2 / (2 * a) ** 2
    E = a * x + b
    return np.array([[pref * np.sum(w * ko.fermi_distribution(E, mu, T))
                      for mu in mus] for T in temps])


def test_conductivity_mixed_bf16x3(kpm):
    """Mixed precision (complex64 recursions, BF16x3 tensor-core moments
    matrix) against the reference's conductivity fixture.  The moments
    matrix is held to 1e-4 relative; sigma, which weights the integrand by
    (1 - e^2)^-2 (kwant/kpm.py:623) and so amplifies moment errors most at
    the outermost nodes, must stay within the error that this moments-
    matrix error implies through the (linear) integral, plus the FP64
    post-processing tolerance of test_conductivity_fp64."""
    g = load('conductivity')
    ham = csr(g)
    pos = g['orb_positions']
    kw = dict(rng=0, num_moments=48, num_vectors=4,
              bounds=(g['lmin'], g['lmax']))
    cond = kpm.conductivity(ham, alpha='x', beta='y', positions=pos,
                            precision='mixed', gemm='bf16x3', **kw)
    # moments matrix: complex64 recursion + BF16 hi/lo products, FP32 sums
    assert _rel(cond.moments_matrix, g['mu_xy']) < 1e-4
    vals = np.array([[cond(mu=m, temperature=T) for m in g['mus']]
                     for T in g['temps']])
    ref = g['values_xy']
    bound = _sigma_error_bound(cond.moments_matrix - g['mu_xy'], cond._a,
                               cond._b, 48, g['mus'], g['temps'])
    err = np.abs(vals - ref)
    tol = bound * (1 + 1e-6) + 1e-9 * np.max(np.abs(ref))
    assert np.all(err <= tol), np.max(err / tol)


def test_conductivity_mixed_fp16x3(kpm):
    """gemm='fp16x3': the same tensor-core products on FP16 hi/lo parts.
    Against the reference's conductivity fixture the moments matrix is held
    to 2e-6 relative (the FP16 split alone, emulated in numpy on these
    vectors: 7.2e-8; the BF16 split: 3.9e-6), and sigma to the error that
    this moments-matrix error implies, as for 'bf16x3'."""
    g = load('conductivity')
    ham = csr(g)
    pos = g['orb_positions']
    kw = dict(rng=0, num_moments=48, num_vectors=4,
              bounds=(g['lmin'], g['lmax']))
    cond = kpm.conductivity(ham, alpha='x', beta='y', positions=pos,
                            precision='mixed', gemm='fp16x3', **kw)
    assert _rel(cond.moments_matrix, g['mu_xy']) < 2e-6
    vals = np.array([[cond(mu=m, temperature=T) for m in g['mus']]
                     for T in g['temps']])
    ref = g['values_xy']
    bound = _sigma_error_bound(cond.moments_matrix - g['mu_xy'], cond._a,
                               cond._b, 48, g['mus'], g['temps'])
    err = np.abs(vals - ref)
    tol = bound * (1 + 1e-6) + 1e-9 * np.max(np.abs(ref))
    assert np.all(err <= tol), np.max(err / tol)


def test_tensor_core_contraction_matches_cuda_cores(kpm):
    """The tcgen05 split-BF16 GEMM equals the CUDA-core evaluation of the
    same hi*hi + hi*lo + lo*hi products (FP32 sums in another order), and
    both approximate the FP64 contraction; moment counts cover partial N
    tiles (48), several M tiles (160) and several N tiles (300)."""
    from kwant_gb300 import _lib, lattices
    syst = lattices.rashba_square(12, seed=3)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    pos = syst.orbital_positions()
    vx = ko.velocity(ham, pos, 0)
    vy = ko.velocity(ham, pos, 1)
    n = ham.shape[0]
    rng = np.random.RandomState(5)
    vecs = np.exp(2j * np.pi * rng.random_sample((6, n)))
    # Gershgorin bound: encloses the spectrum, so the recursion stays bounded
    g = float(np.max(np.asarray(abs(ham).sum(axis=1))))
    a, b = ko.rescale_ab(-g, g, 0.05)
    _a = a * (1 - 0.05 / 2)
    a2, b2 = ko.rescale_ab(b - _a, b + _a, 0.05)
    hm = _lib.Handle(ham, a, b, _lib.PREC_MIXED)
    h64 = _lib.Handle(ham, a, b, _lib.PREC_FP64)
    for M in (48, 160, 300):
        mu_tc = _lib.correlator_moments(hm, a2, b2, vx, vy, vecs, M, gemm=1)
        ms, flops = hm.last_gemm()
        assert ms > 0 and flops > 0
        mu_cc = _lib.correlator_moments(hm, a2, b2, vx, vy, vecs, M, gemm=3)
        mu_64 = _lib.correlator_moments(h64, a2, b2, vx, vy, vecs, M, gemm=0)
        assert _rel(mu_tc, mu_cc) < 1e-5, M
        assert _rel(mu_tc, mu_64) < 1e-4, M
        # FP16 hi/lo parts: the same products with 11-bit parts; a numpy
        # emulation of the split on this case gives 7.5e-8 (BF16: 4.3e-6)
        mu_t16 = _lib.correlator_moments(hm, a2, b2, vx, vy, vecs, M, gemm=4)
        mu_c16 = _lib.correlator_moments(hm, a2, b2, vx, vy, vecs, M, gemm=5)
        assert _rel(mu_t16, mu_c16) < 2e-6, M
        assert _rel(mu_t16, mu_64) < 2e-6, M
    # an odd vector count: the store rows are written one value at a time
    v5 = vecs[:5]
    mu_64 = _lib.correlator_moments(h64, a2, b2, vx, vy, v5, 48, gemm=0)
    for gemm, tol in ((1, 1e-4), (4, 2e-6)):
        mu = _lib.correlator_moments(hm, a2, b2, vx, vy, v5, 48, gemm=gemm)
        assert _rel(mu, mu_64) < tol, gemm


def test_tensor_core_accumulation_runs(kpm, monkeypatch):
    """At a large K (Rashba 120 x 120 x 2, R = 16: K = 460,800, ~12,000 per
    CTA) the tensor cores' FP32 accumulation error dominates the moments
    matrix.  Restarting the accumulation every 1024 K elements (default;
    the run's sums go into a master copy in tensor memory) must be several
    times closer to the FP64 contraction than one run per split
    (KPM_TC_RUN=0), in both part formats; the FP64 path and both formats
    see the same vectors."""
    from kwant_gb300 import _lib, lattices
    syst = lattices.rashba_square(120, seed=0)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    pos = syst.orbital_positions()
    vx = ko.velocity(ham, pos, 0)
    vy = ko.velocity(ham, pos, 1)
    n = ham.shape[0]
    vecs = np.exp(2j * np.pi * np.random.RandomState(1)
                  .random_sample((16, n)))
    g = float(np.max(np.asarray(abs(ham).sum(axis=1))))
    a, b = ko.rescale_ab(-g, g, 0.05)
    _a = a * (1 - 0.05 / 2)
    a2, b2 = ko.rescale_ab(b - _a, b + _a, 0.05)
    hm = _lib.Handle(ham, a, b, _lib.PREC_MIXED)
    h64 = _lib.Handle(ham, a, b, _lib.PREC_FP64)
    M = 256
    mu_64 = _lib.correlator_moments(h64, a2, b2, vx, vy, vecs, M, gemm=0)
    for gemm in (1, 4):
        monkeypatch.delenv('KPM_TC_RUN', raising=False)
        err_runs = _rel(_lib.correlator_moments(hm, a2, b2, vx, vy, vecs, M,
                                                gemm=gemm), mu_64)
        monkeypatch.setenv('KPM_TC_RUN', '0')
        err_one = _rel(_lib.correlator_moments(hm, a2, b2, vx, vy, vecs, M,
                                               gemm=gemm), mu_64)
        assert err_runs < 2e-5 and err_runs * 4 < err_one, \
            (gemm, err_runs, err_one)


def test_fp16_contraction_out_of_range_is_reported(kpm):
    """Vector entries above the FP16 range (65504) make the FP16 split
    contraction non-finite: the call reports KPMDiverged (moments written);
    the BF16 split of the same vectors stays finite and accurate."""
    from kwant_gb300 import _lib, lattices
    syst = lattices.rashba_square(8, seed=1)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    pos = syst.orbital_positions()
    vx = ko.velocity(ham, pos, 0)
    vy = ko.velocity(ham, pos, 1)
    n = ham.shape[0]
    vecs = 1e5 * np.exp(2j * np.pi * np.random.RandomState(2)
                        .random_sample((2, n)))
    g = float(np.max(np.asarray(abs(ham).sum(axis=1))))
    a, b = ko.rescale_ab(-g, g, 0.05)
    _a = a * (1 - 0.05 / 2)
    a2, b2 = ko.rescale_ab(b - _a, b + _a, 0.05)
    hm = _lib.Handle(ham, a, b, _lib.PREC_MIXED)
    with pytest.raises(_lib.KPMDiverged, match='FP16'):
        _lib.correlator_moments(hm, a2, b2, vx, vy, vecs, 32, gemm=4)
    h64 = _lib.Handle(ham, a, b, _lib.PREC_FP64)
    mu_bf = _lib.correlator_moments(hm, a2, b2, vx, vy, vecs, 32, gemm=1)
    mu_64 = _lib.correlator_moments(h64, a2, b2, vx, vy, vecs, 32, gemm=0)
    assert np.all(np.isfinite(mu_bf)) and _rel(mu_bf, mu_64) < 1e-4


# --------------------------------------------------------------- reordering
def test_reordered_handle_parity(kpm):
    """KPM_FLAG_REORDER (RCM storage order) leaves results within rounding
    and keeps the add_vectors bit-identity."""
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Density
    g = load('square100')
    sd = _sd(kpm, csr(g), g, num_moments=100, num_vectors=10, reorder=True)
    assert _rel(np.array(sd._moments_list), g['moments_list']) < TOL
    assert _rel(sd.densities, g['densities']) < TOL
    g = load('honeycomb_ldos')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 1, 0), (n, 0, n)], np.zeros((n, 2)))
    dens = Density(syst, where=list(g['where']))
    sd = _sd(kpm, ham, g, operator=dens, num_moments=60, num_vectors=4,
             reorder=True)
    assert _rel(sd.densities, g['densities']) < TOL
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=5, reorder=True)
    sd.add_vectors(3)
    fresh = _sd(kpm, g['ham'], g, num_moments=200, num_vectors=8,
                reorder=True)
    assert np.array_equal(sd.densities, fresh.densities)
    assert _rel(np.array(sd._moments_list), g['vec_moments_list']) < TOL
    c = load('conductivity')
    cond = kpm.conductivity(csr(c), alpha='x', beta='y',
                            positions=c['orb_positions'], rng=0,
                            num_moments=48, num_vectors=4,
                            bounds=(c['lmin'], c['lmax']), reorder=True)
    assert _rel(cond.moments_matrix, c['mu_xy']) < 1e-11


def test_state_download_matches_oracle(kpm):
    """_last_two_alphas (device state) equals the oracle's recursion."""
    g = load('rmt20')
    sd = _sd(kpm, g['ham'], g, num_moments=10, num_vectors=2, reorder=True)
    _, vecs = ref_vectors(g['seed'], 20, 2)
    a, b = ko.rescale_ab(g['lmin'], g['lmax'], 0.05)
    for r, (prev, cur) in enumerate(sd._last_two_alphas):
        _, (p_ref, c_ref) = ko.moments_dos(g['ham'], a, b, vecs[r], 10)
        assert _rel(prev, p_ref) < 1e-13 and _rel(cur, c_ref) < 1e-13


# ------------------------------------------------------------- determinism
def test_repeatable(kpm):
    g = load('square100')
    a = _sd(kpm, csr(g), g, num_moments=50, num_vectors=10, precision='mixed')
    b = _sd(kpm, csr(g), g, num_moments=50, num_vectors=10, precision='mixed')
    assert np.array_equal(a.densities, b.densities)


def test_call_at_arbitrary_energies_on_device(kpm):
    """SpectralDensity.__call__(energy) (kwant/kpm.py:263-295): the
    Chebyshev sum runs on the device with numpy's Clenshaw arithmetic."""
    from numpy.polynomial.chebyshev import chebval
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Density
    g = load('rashba_ops')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 2, 0), (n // 2, 0, n)], g['positions'])
    rng = np.random.RandomState(3)
    for op in (None, Density(syst, onsite=np.diag([1.0, -1.0]),
                             where=list(g['where_sites']))):
        sd = _sd(kpm, ham, g, operator=op, num_moments=40, num_vectors=3)
        lo, hi = sd.bounds
        E = rng.uniform(lo + 0.1, hi - 0.1, size=(3, 7))
        got = sd(E)
        e = (E - sd._b) / sd._a
        g_e = np.pi * np.sqrt(1 - e) * np.sqrt(1 + e)
        mom = sd._moments()
        mom[1:] = 2 * mom[1:]
        ref = np.transpose(chebval(e, mom) / g_e)
        assert got.shape == ref.shape
        assert np.array_equal(got, ref)
        # scalar energy
        assert np.array_equal(sd(float(E[0, 0])),
                              np.transpose(chebval(e[0, 0], mom) / g_e[0, 0]))


def test_correlator_with_local_operators(kpm):
    """Correlator(operator1=Density, operator2=Current) (kwant/kpm.py:557-
    606): the operators act on the vectors through their ACT maps
    (kwant/operator.pyx:561-606); moments matrix against the oracle with the
    same matrices."""
    from kwant_gb300.system import LatticeSystem
    from kwant_gb300.operator import Density, Current, act_matrix
    g = load('rashba_ops')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 2, 0), (n // 2, 0, n)], g['positions'])
    sz = np.diag([1.0, -1.0])
    dens = Density(syst, onsite=sz)
    cur = Current(syst, onsite=sz, where=[tuple(w) for w in g['hop_where']])
    R, M = 3, 24
    rng = np.random.RandomState(9)
    vecs = np.exp(2j * np.pi * rng.random_sample((R, n)))
    corr = kpm.Correlator(ham, operator1=dens, operator2=cur,
                          vector_factory=list(vecs), num_vectors=R,
                          num_moments=M, bounds=(g['lmin'], g['lmax']))
    ref, _, _ = ko.correlator_moments_matrix(
        ham, vecs, g['lmin'], g['lmax'], M, act_matrix(dens, n),
        act_matrix(cur, n))
    assert _rel(corr.moments_matrix, ref) < 1e-11
