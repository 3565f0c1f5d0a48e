"""Array-backed finite systems for the KPM path.

``LatticeSystem`` holds exactly what the KPM path consumes from a
``kwant.system.FiniteSystem`` (kwant/system.py:20-53, :103-238): the
Hamiltonian as CSR (orbital indices), ``site_ranges``
(kwant/builder.py:703-726 format: rows ``(first_site, norbs, orb_offset)``
plus the terminating ``(num_sites, 0, tot_norbs)``), site positions, and the
site graph.  It is built directly from arrays (see ``kwant_gb300.lattices``)
instead of per-element Python value functions, which is what makes systems
with 10^6-10^7 orbitals constructible in seconds.

It is also what ``kwant_gb300.operator.Density``/``Current`` need: the graph
(edge order), ``site_ranges`` and ``hamiltonian(i, j)`` blocks.
"""

import numpy as np
import scipy.sparse as sp

__all__ = ['LatticeSystem', 'SiteGraph', 'HamiltonianFamily']


class SiteGraph:
    """Compressed site adjacency (kwant/graph/core.pyx CGraph subset).

    Edges are iterated tail-major with heads ascending, matching the
    compressed-graph iteration order of kwant/graph/core.pyx:339-370 for
    graphs whose heads were inserted in sorted order.
    """

    def __init__(self, num_nodes, heads_idxs, heads):
        self.num_nodes = int(num_nodes)
        self.heads_idxs = np.asarray(heads_idxs, dtype=np.int64)
        self.heads = np.asarray(heads, dtype=np.int32)
        self.num_edges = int(self.heads.shape[0])

    def edges(self):
        """All edges as an (E, 2) int32 array (tail, head)."""
        tails = np.repeat(np.arange(self.num_nodes, dtype=np.int32),
                          np.diff(self.heads_idxs))
        return np.stack([tails, self.heads], axis=1)

    def __iter__(self):
        for t, h in self.edges():
            yield (int(t), int(h))

    def out_neighbors(self, node):
        return self.heads[self.heads_idxs[node]:self.heads_idxs[node + 1]]

    def has_edge(self, tail, head):
        if not (0 <= tail < self.num_nodes and 0 <= head < self.num_nodes):
            return False
        nb = self.out_neighbors(tail)
        i = np.searchsorted(nb, head)
        return bool(i < len(nb) and nb[i] == head)


class LatticeSystem:
    """A finite tight-binding system given by arrays.

    Parameters
    ----------
    ham : scipy.sparse matrix (tot_norbs x tot_norbs), Hermitian.
    site_ranges : sequence of (first_site, norbs, orb_offset) triples,
        terminated by (num_sites, 0, tot_norbs).
    positions : (num_sites, dim) float array of site positions.
    """

    def __init__(self, ham, site_ranges, positions, name=''):
        ham = sp.csr_matrix(ham)
        self._ham = ham
        self.site_ranges = [tuple(int(x) for x in r) for r in site_ranges]
        self.positions = np.asarray(positions, dtype=float)
        self.name = name
        sr = np.asarray(self.site_ranges, dtype=np.int64)
        num_sites = int(sr[-1, 0])
        tot = int(sr[-1, 2])
        if ham.shape != (tot, tot):
            raise ValueError('Hamiltonian shape does not match site_ranges')
        if self.positions.shape[0] != num_sites:
            raise ValueError('positions must have one row per site')
        self._orb_site = self._orbital_to_site(sr, tot)
        self.graph = self._site_graph(num_sites)
        self.parameters = frozenset()

    # -- structure ---------------------------------------------------------
    @staticmethod
    def _orbital_to_site(sr, tot):
        site_of = np.empty(tot, dtype=np.int64)
        for k in range(len(sr) - 1):
            first, norbs, off = sr[k]
            last = sr[k + 1, 0]
            n = (last - first) * norbs
            site_of[off:off + n] = first + np.arange(n) // max(norbs, 1)
        return site_of

    def _site_graph(self, num_sites):
        coo = self._ham.tocoo()
        ts = self._orb_site[coo.row]
        hs = self._orb_site[coo.col]
        keep = ts != hs
        pairs = np.unique(np.stack([ts[keep], hs[keep]], axis=1), axis=0)
        counts = np.bincount(pairs[:, 0], minlength=num_sites)
        idx = np.concatenate([[0], np.cumsum(counts)])
        return SiteGraph(num_sites, idx, pairs[:, 1])

    @property
    def num_orbitals(self):
        return int(self.site_ranges[-1][2])

    def pos(self, i):
        return self.positions[i]

    def site_orbitals(self, sites):
        """First orbital and number of orbitals of each site."""
        sr = np.asarray(self.site_ranges, dtype=np.int64)
        sites = np.asarray(sites, dtype=np.int64)
        run = np.searchsorted(sr[:, 0], sites, side='right') - 1
        norbs = sr[run, 1]
        return sr[run, 2] + (sites - sr[run, 0]) * norbs, norbs

    def orbital_positions(self):
        """Position of every orbital (kwant/kpm.py:1072-1073)."""
        return self.positions[self._orb_site]

    # -- kwant.system.System interface subset ------------------------------
    def hamiltonian_submatrix(self, args=(), sparse=False,
                              return_norb=False, *, params=None):
        ham = self._ham.copy() if sparse else self._ham.toarray()
        if sparse:
            ham = ham.tocoo()
        if return_norb:
            sr = np.asarray(self.site_ranges, dtype=np.int64)
            norbs = np.repeat(sr[:-1, 1], np.diff(sr[:, 0]))
            return ham, norbs, norbs
        return ham

    def hamiltonian(self, i, j, *args, params=None):
        si, ni = self.site_orbitals([i])
        sj, nj = self.site_orbitals([j])
        blk = self._ham[si[0]:si[0] + ni[0], sj[0]:sj[0] + nj[0]].toarray()
        if ni[0] == 1 and nj[0] == 1:
            return complex(blk[0, 0])
        return blk

    def hamiltonian_blocks(self, pairs):
        """Dense (a_norbs x b_norbs) blocks for many (a, b) site pairs at
        once, as a list of arrays (vectorised per uniform-norbs group)."""
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        sa, na = self.site_orbitals(pairs[:, 0])
        sb, nb = self.site_orbitals(pairs[:, 1])
        out = [None] * len(pairs)
        csr = self._ham
        for (ua, ub) in set(zip(na.tolist(), nb.tolist())):
            sel = np.nonzero((na == ua) & (nb == ub))[0]
            rows = (sa[sel][:, None, None] + np.arange(ua)[None, :, None])
            cols = (sb[sel][:, None, None] + np.arange(ub)[None, None, :])
            rows, cols = np.broadcast_arrays(rows, cols)
            vals = np.asarray(csr[rows.ravel(), cols.ravel()]).reshape(
                len(sel), ua, ub)
            for k, w in enumerate(sel):
                out[w] = vals[k]
        return out


class HamiltonianFamily:
    """A three-parameter Hamiltonian family on one sparsity structure,

        H(phi, s1, s2) = base .* exp(1j * phi * theta) + s1 * d1 + s2 * d2,

    e.g. hoppings with Peierls phases ``theta`` per unit flux ``phi`` and two
    onsite terms (a fixed disorder pattern of strength ``s1``, a staggered
    mass ``s2``).  The four matrices are scipy CSR with identical
    ``indptr``/``indices`` (entries that vanish at some points are kept as
    explicit zeros); ``theta`` is real.  ``names`` labels the parameters.
    The sweep path (``kwant_gb300.surrogate``) keeps the four matrices on the
    device and regenerates H on the device per point.
    """

    def __init__(self, base, theta, d1, d2, names=('phi', 's1', 's2'),
                 name='family'):
        mats = [sp.csr_matrix(m, dtype=complex) for m in (base, theta, d1, d2)]
        for m in mats:
            m.sort_indices()
        ref = mats[0]
        for m in mats[1:]:
            if (m.shape != ref.shape or
                    not np.array_equal(m.indptr, ref.indptr) or
                    not np.array_equal(m.indices, ref.indices)):
                raise ValueError('family matrices must share one structure')
        if np.any(mats[1].data.imag != 0):
            raise ValueError('theta must be real')
        self.base, self.theta, self.d1, self.d2 = mats
        self.names = tuple(names)
        self.name = name
        self.shape = ref.shape

    def hamiltonian(self, phi, s1, s2):
        """H at one point, on the family's structure (explicit zeros kept)."""
        data = (self.base.data * np.exp(1j * phi * self.theta.data.real) +
                s1 * self.d1.data + s2 * self.d2.data)
        return sp.csr_matrix((data, self.base.indices.copy(),
                              self.base.indptr.copy()), shape=self.shape)

    def gershgorin_bounds(self, box):
        """(lmin, lmax) enclosing the spectrum of every point of the
        parameter box ``((phi_lo, phi_hi), (s1_lo, s1_hi), (s2_lo, s2_hi))``.
        Gershgorin discs with radius sum_j (|base_ij| + |s1 d1_ij + s2
        d2_ij|) off the diagonal; the phase leaves |base| unchanged and the
        rest is linear in (s1, s2), so the corners of the box bound it."""
        n = self.shape[0]
        rows = np.repeat(np.arange(n), np.diff(self.base.indptr))
        diag = rows == self.base.indices
        fixed_diag = diag & (self.theta.data.real == 0)
        b = self.base.data
        lo, hi = np.full(n, np.inf), np.full(n, -np.inf)
        for s1 in box[1]:
            for s2 in box[2]:
                v = s1 * self.d1.data + s2 * self.d2.data
                rad = np.where(diag, 0.0, np.abs(v)) + \
                    np.where(fixed_diag, 0.0, np.abs(b))
                cen = np.where(diag, v.real, 0.0) + \
                    np.where(fixed_diag, b.real, 0.0)
                r = np.bincount(rows, weights=rad, minlength=n)
                c = np.bincount(rows, weights=cen, minlength=n)
                lo = np.minimum(lo, c - r)
                hi = np.maximum(hi, c + r)
        return float(lo.min()), float(hi.max())
