"""Vectorised Hamiltonian assembly for the lattice models of the KPM workloads.

Replaces, for lattices with array-valued onsites and hoppings, the per-element
Python value-function assembly of the reference
(``hamiltonian_submatrix`` -> ``make_sparse_full``, kwant/_system.pyx:94-153
and :233-338).  Conventions match what ``kwant.Builder`` + ``finalized()``
produce for the same model:

* site order: by family, then by tag (kwant/builder.py:2178); a Monatomic
  lattice with tags (x, y) gives index ``x * ny + y``;
* ``H[i, j]`` is the hopping *to* site i *from* site j, ``H[j, i]`` its
  Hermitian conjugate (kwant/builder.py:2049-2100);
* exact zeros are dropped (kwant/_system.pyx:129, :145);
* site positions are ``tag . prim_vecs + offset`` (kwant/lattice.py:501-503).

The model conventions that are free choices (Peierls gauge, Gamma matrices)
are stated in each function's docstring; ``tests/golden/make_golden.py``
builds small twins of each model with ``kwant.Builder`` and the tests check
that the CSR matrices agree.
"""

import numpy as np
import scipy.sparse as sp

from .system import LatticeSystem, HamiltonianFamily

__all__ = ['square', 'honeycomb', 'honeycomb_family', 'rashba_square',
           'wilson_dirac_cubic', 'peierls_phase']

SQRT3 = np.sqrt(3)


def _assemble(n_orbs, rows, cols, vals):
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    vals = np.concatenate(vals).astype(complex)
    keep = vals != 0
    m = sp.coo_matrix((vals[keep], (rows[keep], cols[keep])),
                      shape=(n_orbs, n_orbs))
    m = m.tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return m


def _uniform_site_ranges(n_sites, norbs):
    return [(0, norbs, 0), (n_sites, 0, n_sites * norbs)]


def square(L, W=None, t=-1.0, disorder=(-0.5, 0.5), seed=0):
    """Square lattice L x W, one orbital, nearest-neighbour hopping ``t``,
    onsite Anderson disorder ``U[disorder)`` drawn as
    ``RandomState(seed).uniform(lo, hi, size=(L, W))`` with entry [x, y] on
    site (x, y).  (The 100 x 100 case is the plain-KPM DOS workload.)"""
    W = L if W is None else W
    n = L * W
    x, y = np.divmod(np.arange(n), W)
    lo, hi = disorder
    dis = np.random.RandomState(seed).uniform(lo, hi, size=(L, W)).ravel()
    rows, cols, vals = [np.arange(n)], [np.arange(n)], [dis]
    for dx, dy in ((1, 0), (0, 1)):
        ok = (x + dx < L) & (y + dy < W)
        src = np.nonzero(ok)[0]
        dst = (x[ok] + dx) * W + (y[ok] + dy)
        rows += [dst, src]
        cols += [src, dst]
        vals += [np.full(len(src), t, complex),
                 np.full(len(src), np.conj(t), complex)]
    H = _assemble(n, rows, cols, vals)
    pos = np.stack([x, y], axis=1).astype(float)
    return LatticeSystem(H, _uniform_site_ranges(n, 1), pos,
                         name='square%dx%d' % (L, W))


def peierls_phase(r_to, r_from, flux_per_cell, cell_area):
    """Landau-gauge Peierls phase of the hopping from ``r_from`` to ``r_to``
    for a uniform perpendicular field, A = (-B y, 0):
    phi = -pi * beta * (x_to - x_from) * (y_to + y_from), with
    beta = flux_per_cell / cell_area flux quanta per unit area.
    Antisymmetric under exchange, so H = H^dagger."""
    beta = flux_per_cell / cell_area
    return -np.pi * beta * ((r_to[..., 0] - r_from[..., 0]) *
                            (r_to[..., 1] + r_from[..., 1]))


def _honeycomb_positions(n):
    i, j = np.divmod(np.arange(n * n), n)
    # kwant.lattice.honeycomb(): prim_vecs ((1, 0), (1/2, sqrt(3)/2)),
    # basis offsets (0, 0) and (0, 1/sqrt(3)) (kwant/lattice.py:755-767).
    x = i * 1.0 + j * 0.5
    y = i * 0.0 + j * (0.5 * SQRT3)
    pa = np.stack([x + 0.0, y + 0.0], axis=1)
    pb = np.stack([x + 0.0, y + 1 / SQRT3], axis=1)
    return i, j, pa, pb


def honeycomb(n, t=1.0, flux=0.0, W=0.0, mass=0.0, seed=0):
    """Graphene flake of n x n unit cells (2 n^2 sites, one orbital).

    Sites a(i, j) then b(i, j), 0 <= i, j < n (family a sorts before b);
    nearest-neighbour hopping ``t`` between a(i, j) and b(i, j), b(i, j-1),
    b(i+1, j-1), times the Peierls phase ``exp(1j * peierls_phase(r_to,
    r_from, flux, sqrt(3)/2))`` (``flux`` flux quanta per hexagon);
    onsite ``+mass`` on a, ``-mass`` on b, plus Anderson disorder
    ``RandomState(seed).uniform(-W/2, W/2, size=2 n^2)`` in site order
    (drawn only when W > 0).
    """
    i, j, pa, pb = _honeycomb_positions(n)
    n2 = n * n
    N = 2 * n2
    onsite = np.concatenate([np.full(n2, float(mass)),
                             np.full(n2, -float(mass))])
    if W > 0:
        onsite = onsite + np.random.RandomState(seed).uniform(
            -W / 2, W / 2, size=N)
    rows, cols, vals = [np.arange(N)], [np.arange(N)], [onsite]
    pos = np.concatenate([pa, pb])
    cell = 0.5 * SQRT3
    for di, dj in ((0, 0), (0, -1), (1, -1)):
        ib, jb = i + di, j + dj
        ok = (ib >= 0) & (ib < n) & (jb >= 0) & (jb < n)
        a_idx = np.nonzero(ok)[0]
        b_idx = n2 + ib[ok] * n + jb[ok]
        ph = peierls_phase(pos[a_idx], pos[b_idx], flux, cell) \
            if flux else np.zeros(len(a_idx))
        h_ab = t * np.exp(1j * ph)             # H[a, b]: from b to a
        rows += [a_idx, b_idx]
        cols += [b_idx, a_idx]
        vals += [h_ab, np.conj(h_ab)]
    H = _assemble(N, rows, cols, vals)
    return LatticeSystem(H, [(0, 1, 0), (N, 0, N)], pos,
                         name='honeycomb%d' % n)


def honeycomb_family(n, t=1.0, seed=0):
    """The ``honeycomb`` flake as a family over (flux, W, mass):
    ``family.hamiltonian(flux, W, mass)`` equals ``honeycomb(n, t, flux, W,
    mass, seed).hamiltonian`` up to explicit zeros and rounding (the
    disorder pattern ``u - 1/2`` with ``u = RandomState(seed).uniform(0, 1,
    2 n^2)`` is scaled by W, the Peierls phases per unit flux by flux).
    Every onsite and hopping entry is kept in the structure."""
    i, j, pa, pb = _honeycomb_positions(n)
    n2 = n * n
    N = 2 * n2
    pos = np.concatenate([pa, pb])
    cell = 0.5 * SQRT3
    u = np.random.RandomState(seed).uniform(0.0, 1.0, size=N)
    diag = np.arange(N)
    rows, cols = [diag], [diag]
    base, theta = [np.zeros(N, complex)], [np.zeros(N)]
    dis = [u - 0.5]
    mass = [np.concatenate([np.ones(n2), -np.ones(n2)])]
    for di, dj in ((0, 0), (0, -1), (1, -1)):
        ib, jb = i + di, j + dj
        ok = (ib >= 0) & (ib < n) & (jb >= 0) & (jb < n)
        a_idx = np.nonzero(ok)[0]
        b_idx = n2 + ib[ok] * n + jb[ok]
        th = peierls_phase(pos[a_idx], pos[b_idx], 1.0, cell)
        rows += [a_idx, b_idx]
        cols += [b_idx, a_idx]
        base += [np.full(len(a_idx), t, complex)] * 2
        theta += [th, -th]
        dis += [np.zeros(len(a_idx))] * 2
        mass += [np.zeros(len(a_idx))] * 2
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    indptr = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=N))])
    mats = []
    for vals in (base, theta, dis, mass):
        v = np.concatenate(vals).astype(complex)[order]
        mats.append(sp.csr_matrix((v, c.astype(np.int32), indptr),
                                  shape=(N, N)))
    return HamiltonianFamily(*mats, names=('flux', 'W', 'mass'),
                             name='honeycomb%d' % n)


SIGMA0 = np.eye(2, dtype=complex)
SIGMAX = np.array([[0, 1], [1, 0]], dtype=complex)
SIGMAY = np.array([[0, -1j], [1j, 0]], dtype=complex)
SIGMAZ = np.array([[1, 0], [0, -1]], dtype=complex)


def _block_assemble(n_sites, norbs, rows, cols, blocks):
    """Expand site-level (row, col, norbs x norbs block) triples to orbital
    COO entries and assemble."""
    rr, cc, vv = [], [], []
    oi, oj = np.meshgrid(np.arange(norbs), np.arange(norbs), indexing='ij')
    for r, c, b in zip(rows, cols, blocks):
        b = np.asarray(b, complex)
        if b.ndim == 2:
            b = np.broadcast_to(b, (len(r),) + b.shape)
        rr.append((r[:, None, None] * norbs + oi[None]).ravel())
        cc.append((c[:, None, None] * norbs + oj[None]).ravel())
        vv.append(b.reshape(len(r), norbs, norbs).ravel())
    return _assemble(n_sites * norbs, rr, cc, vv)


def rashba_square(L, t=1.0, alpha=0.3, exchange=0.2, W=1.0, seed=0):
    """Square lattice L x L, two orbitals (spin), the Kubo-Bastin workload.

    onsite = exchange * sigma_z + w_i * sigma_0, w ~ RandomState(seed)
    .uniform(-W/2, W/2, size=L*L) in site order;
    H[(x+1, y), (x, y)] = -t sigma_0 + 1j alpha sigma_y,
    H[(x, y+1), (x, y)] = -t sigma_0 - 1j alpha sigma_x
    (and Hermitian conjugates)."""
    n = L * L
    x, y = np.divmod(np.arange(n), L)
    w = np.random.RandomState(seed).uniform(-W / 2, W / 2, size=n)
    onsite = exchange * SIGMAZ[None] + w[:, None, None] * SIGMA0[None]
    rows, cols, blocks = [np.arange(n)], [np.arange(n)], [onsite]
    hops = {(1, 0): -t * SIGMA0 + 1j * alpha * SIGMAY,
            (0, 1): -t * SIGMA0 - 1j * alpha * SIGMAX}
    for (dx, dy), h in hops.items():
        ok = (x + dx < L) & (y + dy < L)
        src = np.nonzero(ok)[0]
        dst = (x[ok] + dx) * L + (y[ok] + dy)
        rows += [dst, src]
        cols += [src, dst]
        blocks += [h, h.conj().T]
    H = _block_assemble(n, 2, rows, cols, blocks)
    pos = np.stack([x, y], axis=1).astype(float)
    return LatticeSystem(H, [(0, 2, 0), (n, 0, 2 * n)], pos,
                         name='rashba%d' % L)


# Dirac representation used by the Wilson-Dirac model:
# Gamma_0 = tau_z (x) sigma_0, Gamma_j = tau_x (x) sigma_j.
GAMMA0 = np.kron(SIGMAZ, SIGMA0)
GAMMAS = [np.kron(SIGMAX, s) for s in (SIGMAX, SIGMAY, SIGMAZ)]


def wilson_dirac_cubic(L, m=1.5, W=0.0, seed=0):
    """Cubic L^3 lattice, four orbitals: onsite (m - 3) Gamma_0 + w_i 1,
    hopping H[r + e_j, r] = (Gamma_0 - 1j Gamma_j) / 2 (open boundaries),
    w ~ RandomState(seed).uniform(-W/2, W/2, size=L^3) in site order
    (tags (x, y, z) -> index (x L + y) L + z)."""
    n = L ** 3
    idx = np.arange(n)
    x, rem = np.divmod(idx, L * L)
    y, z = np.divmod(rem, L)
    w = np.random.RandomState(seed).uniform(-W / 2, W / 2, size=n) \
        if W > 0 else np.zeros(n)
    onsite = (m - 3) * GAMMA0[None] + w[:, None, None] * np.eye(4)[None]
    rows, cols, blocks = [idx], [idx], [onsite]
    coords = (x, y, z)
    for jdir in range(3):
        d = [0, 0, 0]
        d[jdir] = 1
        ok = (x + d[0] < L) & (y + d[1] < L) & (z + d[2] < L)
        src = np.nonzero(ok)[0]
        dst = ((x[ok] + d[0]) * L + (y[ok] + d[1])) * L + (z[ok] + d[2])
        h = (GAMMA0 - 1j * GAMMAS[jdir]) / 2
        rows += [dst, src]
        cols += [src, dst]
        blocks += [h, h.conj().T]
    H = _block_assemble(n, 4, rows, cols, blocks)
    pos = np.stack(coords, axis=1).astype(float)
    return LatticeSystem(H, [(0, 4, 0), (n, 0, 4 * n)], pos,
                         name='wilson_dirac%d' % L)
