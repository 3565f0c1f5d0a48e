"""Behaviour of the SpectralDensity API on the device, modelled on the
reference's API tests (kwant/tests/test_kpm.py: argument errors,
energy_resolution, custom and local vector factories, convergence) plus
edge sizes (one vector, two moments, odd moment counts, row counts that are
not multiples of the launch granularity, vector counts just above a vector
group) against the CPU oracle."""

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def kpm():
    from kwant_gb300 import kpm
    return kpm


def _herm(n, seed, density=None):
    rng = np.random.RandomState(seed)
    if density is None:
        a = rng.randn(n, n) + 1j * rng.randn(n, n)
        return sp.csr_matrix((a + a.conj().T) / 2)
    a = sp.random(n, n, density=density, random_state=rng) * (1 + 1j)
    a = a + sp.identity(n) * 0.1
    return sp.csr_matrix((a + a.conj().T) / 2)


def test_argument_errors(kpm):
    ham = _herm(20, 0)
    with pytest.raises(ValueError):
        kpm.SpectralDensity('not a hamiltonian')
    with pytest.raises(ValueError):
        kpm.SpectralDensity(ham, operator='not an operator')
    with pytest.raises(ValueError):
        kpm.SpectralDensity(sp.identity(20, dtype=complex, format='csr'))
    with pytest.raises(TypeError):
        kpm.SpectralDensity(ham, num_moments=10, energy_resolution=0.1)
    s = kpm.SpectralDensity(ham, rng=0)
    with pytest.raises(TypeError):
        s.add_moments(num_moments=20, energy_resolution=0.1)
    for v in (-20, 0, 10.5):
        for p in ('num_vectors', 'num_moments'):
            with pytest.raises(ValueError):
                kpm.SpectralDensity(ham, rng=0, **{p: v})
        s = kpm.SpectralDensity(ham, rng=0)
        with pytest.raises(ValueError):
            s.add_moments(num_moments=v)
        with pytest.raises(ValueError):
            s.add_vectors(num_vectors=v)
    for v in (-1, -0.5, 0):
        with pytest.raises(ValueError):
            kpm.SpectralDensity(ham, rng=0, eps=v)
        s = kpm.SpectralDensity(ham, rng=0)
        with pytest.raises(ValueError):
            s.add_moments(energy_resolution=v)
    with pytest.raises(ValueError):
        s.add_moments(energy_resolution=10)      # coarser than present
    s = kpm.SpectralDensity(ham, rng=0, num_vectors=2,
                            accumulate_vectors=False)
    with pytest.raises(ValueError):
        s.add_moments(10)


def test_energy_resolution_equals_num_moments(kpm):
    ham = _herm(30, 1)
    s1 = kpm.SpectralDensity(ham, rng=1, energy_resolution=0.05)
    s2 = kpm.SpectralDensity(ham, rng=1, num_moments=s1.num_moments)
    assert np.array_equal(s1.densities, s2.densities)
    s1.add_moments(energy_resolution=0.03)
    s2.add_moments(s1.num_moments - s2.num_moments)
    assert np.array_equal(s1.densities, s2.densities)


def _exact_moments(ham, a, b, M):
    ev = np.linalg.eigvalsh(ham.toarray())
    x = (ev - b) / a
    return np.cos(np.outer(np.arange(M), np.arccos(x))).sum(axis=1)


def test_local_vectors_give_the_exact_trace(kpm):
    """With one unit vector per orbital the stochastic trace is exact: the
    moments equal sum_k T_n(E_k) from the eigenvalues."""
    ham = _herm(24, 2)
    n = ham.shape[0]
    vecs = kpm.LocalVectors(ham)
    for precision, tol in (('fp64', 1e-11), ('mixed', 2e-5)):
        s = kpm.SpectralDensity(ham, vector_factory=kpm.LocalVectors(ham),
                                num_vectors=n, num_moments=64, rng=0,
                                precision=precision)
        total = np.array(s._moments_list).real.sum(axis=0)
        exact = _exact_moments(ham, s._a, s._b, 64)
        assert np.max(np.abs(total - exact)) <= tol * n, precision
    assert len(vecs) == n


def test_custom_vector_factory_matches_oracle(kpm):
    ham = _herm(40, 3, density=0.2)
    rng = np.random.RandomState(5)
    vecs = [np.rint(rng.random_sample(40)) * 2 - 1 for _ in range(6)]
    lmin, lmax = -10.0, 10.0
    s = kpm.SpectralDensity(ham, vector_factory=iter(vecs), num_vectors=6,
                            num_moments=50, bounds=(lmin, lmax))
    a, b = s._a, s._b
    ref = np.array([ko.moments_dos(ham, a, b, v.astype(complex), 50)[0]
                    for v in vecs])
    got = np.array(s._moments_list)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_convergence_with_moments(kpm):
    """The error of the integrated DOS against the exact eigenvalue count
    decreases as moments are added (exact trace with local vectors)."""
    ham = _herm(40, 4)
    ev = np.linalg.eigvalsh(ham.toarray())
    errs = []
    for M in (20, 80, 320):
        s = kpm.SpectralDensity(ham, vector_factory=kpm.LocalVectors(ham),
                                num_vectors=40, num_moments=M, rng=0)
        e = s.energies
        count = s.integrate(lambda E: (E <= e[len(e) // 2]).astype(float))
        exact = np.mean(ev <= e[len(e) // 2])   # local vectors: per orbital
        errs.append(abs(count - exact))
    assert errs[2] < errs[0]


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('N,R,M', [(17, 1, 2), (17, 1, 3), (33, 15, 7),
                                   (33, 17, 8), (200, 33, 41),
                                   (1000, 64, 12)])
def test_edge_sizes_match_oracle(kpm, precision, N, R, M):
    ham = _herm(N, 7 + N, density=min(1.0, 8.0 / N))
    rng = np.random.RandomState(N + R)
    vecs = np.exp(2j * np.pi * rng.random_sample((R, N)))
    g = float(np.max(np.asarray(abs(ham).sum(axis=1))))
    s = kpm.SpectralDensity(ham, vector_factory=list(vecs), num_vectors=R,
                            num_moments=M, bounds=(-g, g),
                            precision=precision)
    a, b = s._a, s._b
    ref = np.array([ko.moments_dos(ham, a, b, v, M)[0] for v in vecs])
    got = np.array(s._moments_list).reshape(R, M)
    tol = 1e-12 if precision == 'fp64' else 1e-5
    assert np.max(np.abs(got - ref)) <= tol * N
    assert s.densities.shape == (2 * M,)


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_doubling_dos_equals_identity_operator(kpm, precision):
    """kwant/tests/test_kpm.py:342-353: the DOS from the doubling identities
    (operator=None) and from the identity operator (one moment per step,
    no doubling) agree: 1e-12 in FP64; in mixed precision the compensated
    DOS step and the plain complex64 operator path agree within the
    latter's rounding (1e-6 of the DOS maximum)."""
    from kwant_gb300 import lattices
    syst = lattices.honeycomb(30, t=1.0, flux=1e-2, W=0.5, seed=1)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    n = ham.shape[0]
    g = float(np.max(np.asarray(abs(ham).sum(axis=1))))
    kw = dict(num_moments=120, num_vectors=6, rng=3, bounds=(-g, g),
              precision=precision)
    dos = kpm.SpectralDensity(ham, **kw)
    ident = kpm.SpectralDensity(ham, operator=sp.identity(n, format='csr'),
                                **kw)
    tol = 1e-12 if precision == 'fp64' else 1e-6
    assert np.array_equal(dos.energies, ident.energies)
    scale = np.max(np.abs(dos.densities))
    assert np.max(np.abs(dos.densities - ident.densities)) < tol * scale


def test_system_sparse_and_dense_hamiltonians_agree(kpm):
    """kwant/tests/test_kpm.py:393-408: the same Hamiltonian given as a
    system, a sparse matrix and a dense array gives the same moments."""
    from kwant_gb300 import lattices
    syst = lattices.square(12, t=1.0, seed=4)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    kw = dict(num_moments=80, num_vectors=4, rng=9)
    a = kpm.SpectralDensity(syst, **kw)
    b = kpm.SpectralDensity(ham, **kw)
    c = kpm.SpectralDensity(ham.toarray(), **kw)
    for other in (b, c):
        assert np.allclose(other._a, a._a, rtol=0, atol=1e-12 * a._a)
        assert np.max(np.abs(np.array(other._moments_list) -
                             np.array(a._moments_list))) < 1e-10
