"""Generate golden fixtures by running the reference ``kwant.kpm``.

Run in the development container (needs the reference sources, Cython and a
C compiler; see ``build_reference.py``)::

    python tests/golden/make_golden.py

Writes ``tests/golden/*.npz``.  Every fixture stores the inputs the GPU path
needs to reproduce the run without the reference (Hamiltonian CSR, raw
spectral bounds, RNG seed, operator data) and the reference's outputs
(per-vector moments, densities, energies, moments matrix, conductivity).
The fixtures are small (< 2 MB each) and are committed.
"""

import os
import sys

import numpy as np
import scipy
import scipy.sparse as sp
from scipy.sparse.linalg import eigsh

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import build_reference  # noqa: E402

kwant = build_reference.import_reference()
from kwant_gb300 import lattices  # noqa: E402


def _csr(m):
    m = sp.csr_matrix(m)
    return dict(H_data=m.data, H_indices=m.indices.astype(np.int32),
                H_indptr=m.indptr.astype(np.int32),
                H_shape=np.array(m.shape))


def _raw_bounds(ham, eps, seed):
    """The (lmin, lmax) the reference's _rescale computes for rng=seed
    (kwant/kpm.py:201-213, :1166-1172)."""
    rng = np.random.RandomState(seed)
    v0 = np.exp(2j * np.pi * rng.random_sample(ham.shape[0]))
    tol = eps / 2
    lmax = eigsh(ham, k=1, which='LA', return_eigenvectors=False, tol=tol,
                 v0=v0)[0]
    lmin = eigsh(ham, k=1, which='SA', return_eigenvectors=False, tol=tol,
                 v0=v0)[0]
    return lmin, lmax


def _sd_state(sd, prefix=''):
    out = {
        'a': sd._a, 'b': sd._b,
        'moments_list': np.array(sd._moments_list),
        'densities': np.asarray(sd.densities),
        'energies': np.asarray(sd.energies),
        'gammas': np.asarray(sd._gammas),
        'num_moments': sd.num_moments,
        'num_vectors': sd.num_vectors,
    }
    return {prefix + k: v for k, v in out.items()}


def _save(name, **arrays):
    arrays['versions'] = np.array(['numpy ' + np.__version__,
                                   'scipy ' + scipy.__version__])
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **arrays)
    print('wrote', path, os.path.getsize(path), 'bytes')


def make_rmt():
    """Dense GUE-like Hamiltonian of the reference's own tests
    (kwant/tests/test_kpm.py:30-35), seeded."""
    np.random.seed(7)
    ham = kwant.rmt.gaussian(20)
    SD = kwant.kpm.SpectralDensity
    sd = SD(ham, rng=1, num_moments=200, num_vectors=5)
    lmin, lmax = _raw_bounds(sp.csr_matrix(ham), 0.05, 1)
    # resume paths: add_moments (even and odd) and add_vectors
    sd_add = SD(ham, rng=1, num_moments=200, num_vectors=5)
    sd_add.add_moments(200)
    sd_odd = SD(ham, rng=1, num_moments=201, num_vectors=5)
    sd_vec = SD(ham, rng=1, num_moments=200, num_vectors=5)
    sd_vec.add_vectors(3)
    # operator path with a dense identity operator (kwant/kpm.py:195)
    sd_op = SD(ham, rng=1, num_moments=200, num_vectors=5,
               operator=np.identity(20))
    # Lorentz kernel and mean=False
    sd_lor = SD(ham, rng=1, num_moments=64, num_vectors=3,
                kernel=kwant.kpm.lorentz_kernel, mean=False)
    e_eval = np.linspace(sd._b - 0.9 * sd._a, sd._b + 0.9 * sd._a, 11)
    _save('rmt20', ham=ham, lmin=lmin, lmax=lmax, seed=1, eps=0.05,
          call_energies=e_eval, call_values=sd(e_eval),
          integrate=sd.integrate(),
          integrate_fermi=sd.integrate(
              lambda e: kwant.kpm.fermi_distribution(e, 0.1, 0.05)),
          **_sd_state(sd), **_sd_state(sd_add, 'add_'),
          **_sd_state(sd_odd, 'odd_'), **_sd_state(sd_vec, 'vec_'),
          **_sd_state(sd_op, 'op_'), **_sd_state(sd_lor, 'lor_'))


def make_square100():
    """Plain-KPM DOS workload: square 100 x 100, t = -1, onsite disorder
    RandomState(0).uniform(-0.5, 0.5), rng = 1, R = 10, M = 100."""
    L = 100
    lat = kwant.lattice.square(norbs=1)
    syst = kwant.Builder()
    dis = np.random.RandomState(0).uniform(-0.5, 0.5, size=(L, L))
    for x in range(L):
        for y in range(L):
            syst[lat(x, y)] = dis[x, y]
    syst[lat.neighbors()] = -1
    fsyst = syst.finalized()
    sd = kwant.kpm.SpectralDensity(fsyst, num_vectors=10, num_moments=100,
                                   rng=1)
    ham = fsyst.hamiltonian_submatrix(sparse=True).tocsr()
    lmin, lmax = _raw_bounds(ham, 0.05, 1)
    _save('square100', lmin=lmin, lmax=lmax, seed=1, eps=0.05,
          **_csr(ham), **_sd_state(sd))


def make_chain_current():
    """kwant/tests/test_kpm.py:432-454: Current on a chain with params."""
    lat = kwant.lattice.chain(norbs=1)
    syst = kwant.Builder()
    for i in range(20):
        syst[lat(i)] = lambda site, pot: pot
    syst[lat.neighbors()] = lambda s1, s2, t: t
    fsyst = syst.finalized()
    params = {'pot': 1, 't': -2}
    cur = kwant.operator.Current(fsyst)
    sd = kwant.kpm.SpectralDensity(fsyst, params=params, operator=cur,
                                   rng=1, num_moments=200, num_vectors=5)
    ham = fsyst.hamiltonian_submatrix(params=params, sparse=True).tocsr()
    lmin, lmax = _raw_bounds(ham, 0.05, 1)
    _save('chain_current', lmin=lmin, lmax=lmax, seed=1, eps=0.05,
          where=np.asarray(cur.where), **_csr(ham), **_sd_state(sd))


def _honeycomb_builder(n, t, flux, W, mass, seed):
    ref = lattices.honeycomb(n, t=t, flux=flux, W=W, mass=mass, seed=seed)
    onsite = ref._ham.diagonal().real
    lat = kwant.lattice.honeycomb(norbs=1)
    syst = kwant.Builder()
    n2 = n * n
    for i in range(n):
        for j in range(n):
            syst[lat.a(i, j)] = onsite[i * n + j]
            syst[lat.b(i, j)] = onsite[n2 + i * n + j]
    cell = 0.5 * np.sqrt(3)

    def hop(s1, s2):
        return t * np.exp(1j * lattices.peierls_phase(
            np.asarray(s1.pos), np.asarray(s2.pos), flux, cell))
    syst[lat.neighbors()] = hop
    return syst.finalized(), ref


def make_honeycomb_ldos():
    """Honeycomb flake with Peierls phase and disorder; LDOS through
    Density(where=disc) and the DOS."""
    fsyst, _ = _honeycomb_builder(8, 1.0, 0.02, 0.5, 0.1, 3)
    where = [i for i, s in enumerate(fsyst.sites)
             if np.linalg.norm(s.pos - np.array([4.0, 3.5])) < 2.5]
    dens = kwant.operator.Density(fsyst, where=where)
    sd = kwant.kpm.SpectralDensity(fsyst, operator=dens, rng=2,
                                   num_moments=60, num_vectors=4)
    sd_dos = kwant.kpm.SpectralDensity(fsyst, rng=2, num_moments=60,
                                       num_vectors=4)
    dens_sum = kwant.operator.Density(fsyst, where=where, sum=True)
    sd_sum = kwant.kpm.SpectralDensity(fsyst, operator=dens_sum, rng=2,
                                       num_moments=60, num_vectors=4)
    ham = fsyst.hamiltonian_submatrix(sparse=True).tocsr()
    lmin, lmax = _raw_bounds(ham, 0.05, 2)
    _save('honeycomb_ldos', lmin=lmin, lmax=lmax, seed=2, eps=0.05,
          where=np.asarray(where, dtype=np.int32), **_csr(ham),
          **_sd_state(sd), **_sd_state(sd_dos, 'dos_'),
          **_sd_state(sd_sum, 'sum_'))


def _rashba_builder(L, t, alpha, exchange, W, seed):
    ref = lattices.rashba_square(L, t=t, alpha=alpha, exchange=exchange,
                                 W=W, seed=seed)
    w = np.random.RandomState(seed).uniform(-W / 2, W / 2, size=L * L)
    lat = kwant.lattice.square(norbs=2)
    s0, sx, sy, sz = (lattices.SIGMA0, lattices.SIGMAX, lattices.SIGMAY,
                      lattices.SIGMAZ)
    syst = kwant.Builder()
    for x in range(L):
        for y in range(L):
            syst[lat(x, y)] = exchange * sz + w[x * L + y] * s0
    syst[kwant.builder.HoppingKind((1, 0), lat, lat)] = -t * s0 + 1j * alpha * sy
    syst[kwant.builder.HoppingKind((0, 1), lat, lat)] = -t * s0 - 1j * alpha * sx
    return syst.finalized(), ref


def make_rashba_ops():
    """Two-orbital system: Density(sigma_z) summed and local, Current with a
    matrix onsite, and the Kubo-Bastin conductivity."""
    fsyst, _ = _rashba_builder(6, 1.0, 0.3, 0.2, 1.0, 5)
    sz = lattices.SIGMAZ
    where_sites = [i for i in range(0, 36, 5)]
    hop_where = [(a, b) for (a, b) in fsyst.graph if a < b][:12]
    dens_sz = kwant.operator.Density(fsyst, onsite=sz, sum=True)
    dens_loc = kwant.operator.Density(fsyst, onsite=sz, where=where_sites)
    cur = kwant.operator.Current(fsyst, onsite=sz, where=hop_where)
    kw = dict(rng=4, num_moments=40, num_vectors=3)
    SD = kwant.kpm.SpectralDensity
    sd_sz = SD(fsyst, operator=dens_sz, **kw)
    sd_loc = SD(fsyst, operator=dens_loc, **kw)
    sd_cur = SD(fsyst, operator=cur, **kw)
    ham = fsyst.hamiltonian_submatrix(sparse=True).tocsr()
    lmin, lmax = _raw_bounds(ham, 0.05, 4)
    # operator __call__ / act on a fixed vector pair
    rs = np.random.RandomState(11)
    bra = rs.randn(ham.shape[0]) + 1j * rs.randn(ham.shape[0])
    ket = rs.randn(ham.shape[0]) + 1j * rs.randn(ham.shape[0])
    _save('rashba_ops', lmin=lmin, lmax=lmax, seed=4, eps=0.05,
          where_sites=np.asarray(where_sites, np.int32),
          hop_where=np.asarray(hop_where, np.int32), **_csr(ham),
          bra=bra, ket=ket,
          dens_loc_call=dens_loc(bra, ket), dens_sz_call=dens_sz(bra, ket),
          dens_sz_self=dens_sz(bra), cur_call=cur(bra, ket),
          dens_loc_act=dens_loc.act(ket), cur_act=cur.act(ket),
          positions=np.array([fsyst.pos(i) for i in range(len(fsyst.sites))]),
          **_sd_state(sd_sz, 'sz_'), **_sd_state(sd_loc, 'loc_'),
          **_sd_state(sd_cur, 'cur_'))


def make_source_ops():
    """Source operator (kwant/operator.pyx:1003-1126) of sigma_x on the
    two-orbital Rashba + exchange system: local and summed, __call__, act,
    and as the operator of a SpectralDensity."""
    fsyst, _ = _rashba_builder(6, 1.0, 0.3, 0.2, 1.0, 5)
    sx = lattices.SIGMAX
    where_sites = [i for i in range(0, 36, 4)]
    src_loc = kwant.operator.Source(fsyst, onsite=sx, where=where_sites)
    src_sum = kwant.operator.Source(fsyst, onsite=sx, sum=True)
    kw = dict(rng=6, num_moments=30, num_vectors=3)
    sd_loc = kwant.kpm.SpectralDensity(fsyst, operator=src_loc, **kw)
    sd_sum = kwant.kpm.SpectralDensity(fsyst, operator=src_sum, **kw)
    ham = fsyst.hamiltonian_submatrix(sparse=True).tocsr()
    lmin, lmax = _raw_bounds(ham, 0.05, 6)
    rs = np.random.RandomState(12)
    bra = rs.randn(ham.shape[0]) + 1j * rs.randn(ham.shape[0])
    ket = rs.randn(ham.shape[0]) + 1j * rs.randn(ham.shape[0])
    _save('source_ops', lmin=lmin, lmax=lmax, seed=6, eps=0.05,
          where_sites=np.asarray(where_sites, np.int32), **_csr(ham),
          bra=bra, ket=ket, loc_call=src_loc(bra, ket),
          sum_call=src_sum(bra, ket), sum_self=src_sum(bra),
          loc_act=src_loc.act(ket), sum_act=src_sum.act(ket),
          **_sd_state(sd_loc, 'loc_'), **_sd_state(sd_sum, 'sum_'))


def make_conductivity():
    """Kubo-Bastin sigma_xy on a small Rashba + exchange system
    (kwant/kpm.py:763-847)."""
    fsyst, _ = _rashba_builder(6, 1.0, 0.3, 0.2, 1.0, 6)
    kw = dict(rng=0, num_moments=48, num_vectors=4)
    cond = kwant.kpm.conductivity(fsyst, alpha='x', beta='y', **kw)
    cond_xx = kwant.kpm.conductivity(fsyst, alpha='x', beta='x', **kw)
    mus = np.linspace(-2.0, 2.0, 9)
    temps = [0.0, 0.1]
    vals = np.array([[cond(mu=m, temperature=T) for m in mus]
                     for T in temps])
    vals_xx = np.array([[cond_xx(mu=m, temperature=T) for m in mus]
                        for T in temps])
    ham = fsyst.hamiltonian_submatrix(sparse=True).tocsr()
    lmin, lmax = _raw_bounds(ham, 0.05, 0)
    norbs = 2
    pos = np.array([fsyst.pos(i) for i in range(len(fsyst.sites))])
    orb_pos = np.repeat(pos, norbs, axis=0)
    # resume: add_moments on an accumulating correlator
    cond_add = kwant.kpm.conductivity(fsyst, alpha='x', beta='y',
                                      accumulate_vectors=True, **kw)
    cond_add.add_moments(16)
    vals_add = np.array([cond_add(mu=m, temperature=0.1) for m in mus])
    _save('conductivity', lmin=lmin, lmax=lmax, seed=0, eps=0.05,
          **_csr(ham), orb_positions=orb_pos, mus=mus,
          temps=np.array(temps), values_xy=vals, values_xx=vals_xx,
          mu_xy=cond.moments_matrix, mu_xx=cond_xx.moments_matrix,
          a=cond._a, b=cond._b, factor_xy=cond._integral_factor,
          energies=cond.energies, values_add=vals_add,
          mu_add=cond_add.moments_matrix)


def make_lattice_twins():
    """CSR equality of the vectorised lattice assembly and kwant.Builder."""
    out = {}
    # square
    L, Wd = 5, 4
    lat = kwant.lattice.square(norbs=1)
    syst = kwant.Builder()
    dis = np.random.RandomState(9).uniform(-0.5, 0.5, size=(L, Wd))
    for x in range(L):
        for y in range(Wd):
            syst[lat(x, y)] = dis[x, y]
    syst[lat.neighbors()] = -1
    fs = syst.finalized()
    out.update({'square_' + k: v for k, v in
                _csr(fs.hamiltonian_submatrix(sparse=True)).items()})
    out['square_pos'] = np.array([s.pos for s in fs.sites])
    # honeycomb with flux, mass, disorder
    fs, _ = _honeycomb_builder(5, 1.0, 0.05, 0.5, 0.2, 1)
    out.update({'honeycomb_' + k: v for k, v in
                _csr(fs.hamiltonian_submatrix(sparse=True)).items()})
    out['honeycomb_pos'] = np.array([s.pos for s in fs.sites])
    # rashba
    fs, _ = _rashba_builder(4, 1.0, 0.3, 0.2, 1.0, 2)
    out.update({'rashba_' + k: v for k, v in
                _csr(fs.hamiltonian_submatrix(sparse=True)).items()})
    # wilson-dirac
    Lc, m = 3, 1.5
    latc = kwant.lattice.cubic(norbs=4)
    syst = kwant.Builder()
    w = np.random.RandomState(8).uniform(-1.0, 1.0, size=Lc ** 3)
    for x in range(Lc):
        for y in range(Lc):
            for z in range(Lc):
                syst[latc(x, y, z)] = ((m - 3) * lattices.GAMMA0
                                       + w[(x * Lc + y) * Lc + z] * np.eye(4))
    for j in range(3):
        d = [0, 0, 0]
        d[j] = 1
        syst[kwant.builder.HoppingKind(tuple(d), latc, latc)] = \
            (lattices.GAMMA0 - 1j * lattices.GAMMAS[j]) / 2
    fs = syst.finalized()
    out.update({'wilson_' + k: v for k, v in
                _csr(fs.hamiltonian_submatrix(sparse=True)).items()})
    _save('lattice_twins', **out)


if __name__ == '__main__':
    which = sys.argv[1:] or ['rmt', 'square100', 'chain_current',
                             'honeycomb_ldos', 'rashba_ops', 'conductivity',
                             'lattice_twins', 'source_ops']
    for name in which:
        globals()['make_' + name]()
