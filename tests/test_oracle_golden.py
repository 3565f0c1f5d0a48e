"""Pin the CPU oracle against golden vectors produced by the reference.

These run without a GPU.  They establish that ``oracle/kpm_oracle.py``
reproduces the reference ``kwant.kpm`` on the same inputs, so that the GPU
parity tests can use the oracle at sizes the fixtures do not cover.
"""

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from oracle import kpm_oracle as ko  # noqa: E402

from golden_io import load, csr, ref_vectors  # noqa: E402

TOL = 1e-12


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_rmt_dos_matches_reference():
    g = load('rmt20')
    ham = g['ham']
    n = ham.shape[0]
    _, vecs = ref_vectors(g['seed'], n, 5)
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 200)
    assert out['a'] == g['a'] and out['b'] == g['b']
    assert _rel(out['moments_list'], g['moments_list']) < TOL
    assert _rel(out['densities'], g['densities']) < TOL
    assert np.array_equal(out['energies'], g['energies'])


def test_rmt_resume_and_odd():
    g = load('rmt20')
    ham = g['ham']
    a, b = ko.rescale_ab(g['lmin'], g['lmax'], 0.05)
    _, vecs = ref_vectors(g['seed'], 20, 8)
    for r in range(5):
        m200, st = ko.moments_dos(ham, a, b, vecs[r], 200)
        m400, _ = ko.moments_dos(ham, a, b, vecs[r], 400, state=st, prev=m200)
        assert _rel(m400, g['add_moments_list'][r]) < TOL
        m201, _ = ko.moments_dos(ham, a, b, vecs[r], 201)
        assert _rel(m201, g['odd_moments_list'][r]) < TOL
    # add_vectors: vectors 5..7 continue the same stream
    for r in range(8):
        m, _ = ko.moments_dos(ham, a, b, vecs[r], 200)
        assert _rel(m, g['vec_moments_list'][r]) < TOL


def test_rmt_operator_path_and_kernels():
    g = load('rmt20')
    ham = g['ham']
    _, vecs = ref_vectors(g['seed'], 20, 5)
    ident = np.identity(20)
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 200,
                              op=lambda bra, ket: np.vdot(bra, ident @ ket))
    assert _rel(out['moments_list'], g['op_moments_list']) < TOL
    assert _rel(out['densities'], g['op_densities']) < TOL
    out = ko.spectral_density(ham, vecs[:3], g['lmin'], g['lmax'], 64,
                              mean=False, kernel=ko.lorentz_kernel)
    assert _rel(out['densities'], g['lor_densities']) < TOL


def test_rmt_call_and_integrate():
    g = load('rmt20')
    mom = ko.reduce_moments(g['moments_list'], g['a'])
    vals = ko.evaluate(mom, g['a'], g['b'], g['call_energies'])
    assert _rel(vals, g['call_values']) < TOL
    assert abs(ko.integrate(g['gammas'], g['a'], 200) - g['integrate']) < TOL
    f = ko.integrate(g['gammas'], g['a'], 200, g['energies'],
                     lambda e: ko.fermi_distribution(e, 0.1, 0.05))
    assert abs(f - g['integrate_fermi']) < TOL


def test_square100_dos_matches_reference():
    g = load('square100')
    ham = csr(g)
    _, vecs = ref_vectors(g['seed'], ham.shape[0], 10)
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 100)
    assert out['a'] == g['a'] and out['b'] == g['b']
    assert _rel(out['moments_list'], g['moments_list']) < TOL
    assert _rel(out['densities'], g['densities']) < TOL


def test_ldos_density_operator():
    g = load('honeycomb_ldos')
    ham = csr(g)
    n = ham.shape[0]
    _, vecs = ref_vectors(g['seed'], n, 4)
    sr = [(0, 1, 0), (n, 0, n)]
    where = g['where']
    op = lambda bra, ket: ko.density_matels(bra, ket, sr, where, np.eye(1))
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 60, op=op)
    assert _rel(out['moments_list'], g['moments_list']) < TOL
    assert _rel(out['densities'], g['densities']) < TOL
    op = lambda bra, ket: ko.density_matels(bra, ket, sr, where, np.eye(1),
                                            sum_=True)
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 60, op=op)
    assert _rel(out['densities'], g['sum_densities']) < TOL


def test_current_operator_chain():
    g = load('chain_current')
    ham = csr(g)
    n = ham.shape[0]
    _, vecs = ref_vectors(g['seed'], n, 5)
    sr = [(0, 1, 0), (n, 0, n)]
    where = g['where']
    blocks = [ham[a:a + 1, b:b + 1].toarray() for a, b in where]
    op = lambda bra, ket: ko.current_matels(bra, ket, sr, where, blocks,
                                            np.eye(1))
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 200, op=op)
    assert _rel(out['moments_list'], g['moments_list']) < TOL
    assert _rel(out['densities'], g['densities']) < TOL


def test_two_orbital_operators():
    g = load('rashba_ops')
    ham = csr(g)
    n = ham.shape[0]
    sr = [(0, 2, 0), (n // 2, 0, n)]
    sz = np.diag([1.0, -1.0]).astype(complex)
    bra, ket = g['bra'], g['ket']
    ws = g['where_sites']
    assert _rel(ko.density_matels(bra, ket, sr, ws, sz),
                g['dens_loc_call']) < TOL
    allsites = np.arange(n // 2)
    assert abs(ko.density_matels(bra, ket, sr, allsites, sz, sum_=True)
               - g['dens_sz_call']) < 1e-10
    hw = g['hop_where']
    blocks = [ham[2 * a:2 * a + 2, 2 * b:2 * b + 2].toarray() for a, b in hw]
    assert _rel(ko.current_matels(bra, ket, sr, hw, blocks, sz),
                g['cur_call']) < TOL
    _, vecs = ref_vectors(g['seed'], n, 3)
    op = lambda b_, k_: ko.current_matels(b_, k_, sr, hw, blocks, sz)
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 40, op=op)
    assert _rel(out['densities'], g['cur_densities']) < TOL


def test_source_operator_matches_reference():
    g = load('source_ops')
    ham = csr(g)
    n = ham.shape[0]
    sr = [(0, 2, 0), (n // 2, 0, n)]
    sx = np.array([[0, 1], [1, 0]], complex)
    bra, ket = g['bra'], g['ket']
    ws = g['where_sites']
    blocks = [ham[2 * a:2 * a + 2, 2 * a:2 * a + 2].toarray() for a in ws]
    assert _rel(ko.source_matels(bra, ket, sr, ws, blocks, sx),
                g['loc_call']) < TOL
    allsites = np.arange(n // 2)
    ball = [ham[2 * a:2 * a + 2, 2 * a:2 * a + 2].toarray() for a in allsites]
    assert abs(ko.source_matels(bra, ket, sr, allsites, ball, sx, sum_=True)
               - g['sum_call']) < 1e-10
    assert abs(ko.source_matels(bra, bra, sr, allsites, ball, sx, sum_=True,
                                real=True) - g['sum_self']) < 1e-10
    assert _rel(ko.source_act(ket, sr, ws, blocks, sx), g['loc_act']) < TOL
    _, vecs = ref_vectors(g['seed'], n, 3)
    op = lambda b_, k_: ko.source_matels(b_, k_, sr, ws, blocks, sx)
    out = ko.spectral_density(ham, vecs, g['lmin'], g['lmax'], 30, op=op)
    assert _rel(out['densities'], g['loc_densities']) < TOL


def test_conductivity_matches_reference():
    g = load('conductivity')
    ham = csr(g)
    n = ham.shape[0]
    _, vecs = ref_vectors(g['seed'], n, 4)
    pos = g['orb_positions']
    vx = ko.velocity(ham, pos, 0)
    vy = ko.velocity(ham, pos, 1)
    mu, (a, b), _ = ko.correlator_moments_matrix(
        ham, vecs, g['lmin'], g['lmax'], 48, vx, vy)
    assert a == g['a'] and b == g['b']
    assert _rel(mu, g['mu_xy']) < 1e-11
    fac = ko.integral_factor(mu, a, b, 48)
    assert _rel(fac, g['factor_xy']) < 1e-10
    for it, T in enumerate(g['temps']):
        for im, m in enumerate(g['mus']):
            v = ko.conductivity_value(fac, a, b, 48, m, T)
            assert abs(v - g['values_xy'][it, im]) < 1e-9 * max(
                1, abs(g['values_xy'][it, im]))


@pytest.mark.parametrize('model', ['square', 'honeycomb', 'rashba',
                                   'wilson'])
def test_lattice_assembly_matches_builder(model):
    """Vectorised Hamiltonian assembly == kwant.Builder + finalized()."""
    from kwant_gb300 import lattices
    g = load('lattice_twins')
    ref = csr(g, model + '_')
    if model == 'square':
        ours = lattices.square(5, 4, t=-1, seed=9)
    elif model == 'honeycomb':
        ours = lattices.honeycomb(5, t=1.0, flux=0.05, W=0.5, mass=0.2,
                                  seed=1)
    elif model == 'rashba':
        ours = lattices.rashba_square(4, seed=2)
    else:
        ours = lattices.wilson_dirac_cubic(3, m=1.5, W=2.0, seed=8)
    H = ours.hamiltonian_submatrix(sparse=True).tocsr()
    assert H.shape == ref.shape
    assert H.nnz == ref.nnz
    assert abs(H - ref).max() < 1e-13
    if model + '_pos' in g:
        assert np.allclose(ours.positions, g[model + '_pos'], atol=1e-14)
