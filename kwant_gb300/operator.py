"""Local operators of the KPM path: Density and Current.

Mirrors ``kwant.operator.Density`` / ``Current`` (kwant/operator.pyx:723-1000)
for systems given as :class:`kwant_gb300.system.LatticeSystem` or as a
finalized Kwant system (duck-typed: ``graph``, ``site_ranges``,
``hamiltonian``).  The operators do not evaluate anything on the host:
``__call__`` (MAT_ELS) and ``act`` (ACT) run on the device.  They are
*lowered* to a sesquilinear "term" form that the CUDA library evaluates:

    coef_t = sum_e conj(v_e) bra[col_e]          (bra-side factor of term t)
    q_w    = sum_{t in w} conj(coef_t) ket[row_t]

The same lowering accepts reference ``kwant.operator`` objects
(:func:`lower`), reading their public attributes (kwant/operator.pxd:29-33),
and matrix operators ``vdot(bra, O ket)`` (kwant/kpm.py:195).
"""

import collections.abc
import numbers
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

__all__ = ['Density', 'Current', 'Source', 'lower', 'lower_matrix', 'act_matrix',
           'LoweredOperator']

gint_dtype = np.int32
SUM_CHUNK = 64  # terms per chunk of a summed (scalar) output


@dataclass
class LoweredOperator:
    num_terms: int
    num_outputs: int
    num_chunks: int
    term_row: np.ndarray   # int32 (T,)
    bra_ptr: np.ndarray    # int64 (T+1,)
    bra_col: np.ndarray    # int32 (E,)
    bra_val: np.ndarray    # complex128 (E,)
    chunk_ptr: np.ndarray  # int64 (C+1,)
    chunk_out: np.ndarray  # int32 (C,)
    real0: bool
    scalar: bool           # output is a scalar (sum=True or matrix op)


def _finish(term_row, term_out, bra_ptr, bra_col, bra_val, num_outputs,
            sum_, real0, scalar):
    """Drop empty terms, sort by output, build chunks."""
    term_row = np.asarray(term_row, np.int64)
    term_out = np.asarray(term_out, np.int64)
    bra_ptr = np.asarray(bra_ptr, np.int64)
    bra_col = np.asarray(bra_col, np.int64)
    bra_val = np.asarray(bra_val, complex)
    # drop zero bra entries and terms without entries
    cnt = np.diff(bra_ptr)
    seg = np.repeat(np.arange(len(term_row)), cnt)
    keep_e = bra_val != 0
    seg, bra_col, bra_val = seg[keep_e], bra_col[keep_e], bra_val[keep_e]
    cnt = np.bincount(seg, minlength=len(term_row))
    keep_t = cnt > 0
    new_id = np.cumsum(keep_t) - 1
    term_row, term_out, cnt = term_row[keep_t], term_out[keep_t], cnt[keep_t]
    seg = new_id[seg]
    # stable sort of terms by output
    order = np.argsort(term_out, kind='stable')
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    term_row, term_out, cnt = term_row[order], term_out[order], cnt[order]
    eorder = np.argsort(inv[seg], kind='stable')
    bra_col, bra_val = bra_col[eorder], bra_val[eorder]
    bra_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    T = len(term_row)
    if sum_:
        W = 1
        starts = np.arange(0, T, SUM_CHUNK)
        chunk_ptr = np.concatenate([starts, [T]]).astype(np.int64)
        chunk_out = np.zeros(len(starts), np.int32)
    else:
        W = int(num_outputs)
        if T:
            bnd = np.nonzero(np.diff(term_out))[0] + 1
            starts = np.concatenate([[0], bnd])
            chunk_ptr = np.concatenate([starts, [T]]).astype(np.int64)
            chunk_out = term_out[starts].astype(np.int32)
        else:
            chunk_ptr = np.zeros(1, np.int64)
            chunk_out = np.zeros(0, np.int32)
    return LoweredOperator(
        num_terms=T, num_outputs=W, num_chunks=len(chunk_out),
        term_row=np.ascontiguousarray(term_row, np.int32),
        bra_ptr=bra_ptr, bra_col=np.ascontiguousarray(bra_col, np.int32),
        bra_val=np.ascontiguousarray(bra_val, np.complex128),
        chunk_ptr=chunk_ptr, chunk_out=np.ascontiguousarray(chunk_out),
        real0=bool(real0), scalar=bool(scalar or sum_))


def _site_orbitals(site_ranges, sites):
    """kwant/operator.pyx:114-125 (_get_orbs) for many sites."""
    sr = np.asarray(site_ranges, dtype=np.int64)
    sites = np.asarray(sites, dtype=np.int64)
    run = np.searchsorted(sr[:, 0], sites, side='right') - 1
    norbs = sr[run, 1]
    return sr[run, 2] + (sites - sr[run, 0]) * norbs, norbs


def _blocks_for(mats, norbs):
    """Per-site (n x n) matrices: ``mats`` is a list of matrices or one
    matrix used everywhere.  A unique matrix larger than a site's norbs is
    read the way the reference reads it (flat, row stride norbs:
    kwant/operator.pyx:801-807 with the onsite broadcast of :303-308)."""
    out = []
    for w, n in enumerate(norbs):
        M = mats[w] if isinstance(mats, list) else mats
        M = np.asarray(M, complex)
        if M.ndim == 0:
            M = M.reshape(1, 1)
        if M.shape[0] != n:
            M = M.ravel()[:n * n].reshape(n, n)
        out.append(M)
    return out


def lower_density(site_ranges, where, onsite_mats, sum_=False,
                  check_hermiticity=True):
    """Density MAT_ELS (kwant/operator.pyx:785-807) in term form:
    q_w = sum_j conj(coef_j) ket[s+j], coef_j = sum_i conj(M[i,j]) bra[s+i]."""
    where = np.asarray(where, dtype=np.int64).reshape(-1)
    start, norbs = _site_orbitals(site_ranges, where)
    rows, outs, ptr, cols, vals = [], [], [0], [], []
    uniform = not isinstance(onsite_mats, list)
    if uniform and len(set(norbs.tolist())) <= 1 and len(where):
        n = int(norbs[0])
        M = _blocks_for(onsite_mats, [n])[0]
        W = len(where)
        j = np.arange(n)
        rows = (start[:, None] + j[None, :]).ravel()
        outs = np.repeat(np.arange(W), n)
        # term (w, j) has entries i = 0..n-1: column s_w + i, value M[i, j]
        cols = np.broadcast_to(start[:, None, None] + j[None, None, :],
                               (W, n, n)).ravel()
        vals = np.broadcast_to(M.T[None, :, :], (W, n, n)).ravel()
        ptr = np.arange(0, W * n * n + 1, n)
    else:
        blocks = _blocks_for(onsite_mats, norbs)
        for w in range(len(where)):
            s, n, M = int(start[w]), int(norbs[w]), blocks[w]
            for j in range(n):
                rows.append(s + j)
                outs.append(w)
                for i in range(n):
                    cols.append(s + i)
                    vals.append(M[i, j])
                ptr.append(len(cols))
    return _finish(rows, outs, ptr, cols, vals, len(where), sum_,
                   check_hermiticity, False)


def lower_current(site_ranges, hoppings, hop_blocks, onsite_mats, sum_=False,
                  check_hermiticity=True):
    """Current MAT_ELS (kwant/operator.pyx:977-987) in term form.  For
    hopping (a, b) with H = H_ab (na x nb) and M = M_a:
      J = i [conj(bra_b) H^dag M ket_a - conj(bra_a) M H ket_b]
    terms on ket_a rows: coef_k = sum_i conj(1j (H^dag M)[i,k]) bra_b[i];
    terms on ket_b rows: coef_i = sum_j conj(-1j (M H)[j,i]) bra_a[j]."""
    hoppings = np.asarray(hoppings, dtype=np.int64).reshape(-1, 2)
    a_s, a_n = _site_orbitals(site_ranges, hoppings[:, 0])
    b_s, b_n = _site_orbitals(site_ranges, hoppings[:, 1])
    Ms = _blocks_for(onsite_mats, a_n)
    rows, outs, ptr, cols, vals = [], [], [0], [], []
    for w in range(len(hoppings)):
        H = np.asarray(hop_blocks[w], complex).reshape(a_n[w], b_n[w])
        M = Ms[w]
        A = 1j * (H.conj().T @ M)      # (nb x na): [i, k]
        B = -1j * (M @ H)              # (na x nb): [j, i]
        for k in range(a_n[w]):
            rows.append(a_s[w] + k)
            outs.append(w)
            for i in range(b_n[w]):
                cols.append(b_s[w] + i)
                vals.append(A[i, k])
            ptr.append(len(cols))
        for i in range(b_n[w]):
            rows.append(b_s[w] + i)
            outs.append(w)
            for j in range(a_n[w]):
                cols.append(a_s[w] + j)
                vals.append(B[j, i])
            ptr.append(len(cols))
    return _finish(rows, outs, ptr, cols, vals, len(hoppings), sum_,
                   check_hermiticity, False)


def lower_matrix(op):
    """``vdot(bra, O ket)`` (kwant/kpm.py:193-195): one term per column j
    of O, coef_j = (O^dag bra)_j."""
    O = sp.csc_matrix(op)
    O.sum_duplicates()
    rows = np.arange(O.shape[1])
    return _finish(rows, np.zeros(O.shape[1], np.int64), O.indptr, O.indices,
                   O.data, 1, True, False, True)


# --------------------------------------------------------------------------
# ACT as a sparse matrix (for the correlator's operator application)
# --------------------------------------------------------------------------

def act_matrix(op, n_orbs, params=None):
    """The linear map ``op.act`` as a CSR matrix.  Density ACT
    (kwant/operator.pyx:808-813): out[s+i] += M[i,j] ket[s+j]; Current ACT
    (kwant/operator.pyx:989-1000): out[b_s+i] += 1j (H^dag M)[i,k] ket[a_s+k],
    out[a_s+j] += -1j (M H)[j,i] ket[b_s+i]."""
    info = _operator_info(op, params)
    rows, cols, vals = [], [], []
    if info['kind'] == 'density':
        start, norbs = _site_orbitals(info['site_ranges'], info['where'])
        blocks = _blocks_for(info['onsite'], norbs)
        for w in range(len(start)):
            s, n, M = start[w], norbs[w], blocks[w]
            ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
            rows.append((s + ii).ravel())
            cols.append((s + jj).ravel())
            vals.append(M.ravel())
    else:
        hops = info['where']
        a_s, a_n = _site_orbitals(info['site_ranges'], hops[:, 0])
        b_s, b_n = _site_orbitals(info['site_ranges'], hops[:, 1])
        Ms = _blocks_for(info['onsite'], a_n)
        for w in range(len(hops)):
            H = np.asarray(info['hop_blocks'][w], complex).reshape(
                a_n[w], b_n[w])
            M = Ms[w]
            A = 1j * (H.conj().T @ M)
            B = -1j * (M @ H)
            ii, kk = np.meshgrid(np.arange(b_n[w]), np.arange(a_n[w]),
                                 indexing='ij')
            rows.append((b_s[w] + ii).ravel())
            cols.append((a_s[w] + kk).ravel())
            vals.append(A.ravel())
            jj, ii2 = np.meshgrid(np.arange(a_n[w]), np.arange(b_n[w]),
                                  indexing='ij')
            rows.append((a_s[w] + jj).ravel())
            cols.append((b_s[w] + ii2).ravel())
            vals.append(B.ravel())
    if rows:
        rows = np.concatenate(rows)
        cols = np.concatenate(cols)
        vals = np.concatenate(vals)
    m = sp.coo_matrix((vals, (rows, cols)), shape=(n_orbs, n_orbs))
    return m.tocsr()


# --------------------------------------------------------------------------
# Operator classes
# --------------------------------------------------------------------------

def _normalize_site_where(syst, where):
    """kwant/operator.pyx:160-199 (finite systems)."""
    n_sites = syst.graph.num_nodes
    if where is None:
        where = list(range(n_sites))
    elif callable(where):
        if hasattr(syst, 'sites') and hasattr(syst, 'id_by_site'):
            where = [syst.id_by_site[s] for s in filter(where, syst.sites)]
        else:
            where = [s for s in range(n_sites) if where(s)]
    else:
        if len(where) and not isinstance(where[0], numbers.Integral):
            try:
                where = [syst.id_by_site[s] for s in where]
            except AttributeError:
                raise TypeError("'where' contains Sites, but the system is "
                                "not a finalized Builder.")
    where = np.asarray(where, dtype=gint_dtype).reshape(-1, 1)
    if np.any(np.logical_or(where < 0, where >= n_sites)):
        raise ValueError('`where` contains sites that are not in the '
                         'system.')
    return where


def _normalize_hopping_where(syst, where):
    """kwant/operator.pyx:202-251 (finite systems)."""
    if where is None:
        where = list(syst.graph)
    elif callable(where):
        if hasattr(syst, 'sites'):
            where = [h for h in syst.graph
                     if where(syst.sites[h[0]], syst.sites[h[1]])]
        else:
            where = [h for h in syst.graph if where(*h)]
    else:
        if len(where) and not isinstance(where[0][0], numbers.Integral):
            try:
                where = [(syst.id_by_site[a], syst.id_by_site[b])
                         for a, b in where]
            except AttributeError:
                raise TypeError("'where' contains Sites, but the system is "
                                "not a finalized Builder.")
        if any(not syst.graph.has_edge(*w) for w in where):
            raise ValueError('`where` contains hoppings that are not in the '
                             'system.')
    return np.asarray(where, dtype=gint_dtype).reshape(-1, 2)


def _is_herm(M, rtol=1e-13, atol=1e-300):
    """kwant/operator.pyx:48-73 (_is_herm_conj(M, M))."""
    M = np.asarray(M, complex)
    tol = rtol * np.max(np.abs(M)) + atol
    return np.all(np.abs(M - M.conj().T) ** 2 <= tol)


def _normalize_onsite(syst, onsite, check_hermiticity):
    """kwant/operator.pyx:283-321: returns a matrix or a callable."""
    if callable(onsite):
        return onsite
    if isinstance(onsite, collections.abc.Mapping):
        if not hasattr(syst, 'sites'):
            raise TypeError('Provide `onsite` as a value or a function for '
                            'systems that are not finalized Builders.')
        return onsite
    M = np.asarray(onsite, complex)
    if M.ndim == 0:
        M = M.reshape(1, 1)
    if M.ndim != 2 or M.shape[0] != M.shape[1]:
        raise ValueError('Onsite matrix is not square')
    if check_hermiticity and not _is_herm(M):
        raise ValueError('Onsite matrix is not hermitian, use the option '
                         '`check_hermiticity=True` if this is intentional.')
    if M.shape[0] == 1:
        max_norbs = max(n for (_, n, _) in syst.site_ranges)
        return M[0, 0] * np.identity(max_norbs, complex)
    norbs = set(r[1] for r in syst.site_ranges[:-1])
    if len(norbs) != 1:
        raise ValueError('Single `onsite` matrix provided, but there are '
                         'different numbers of orbitals on different sites')
    if M.shape[0] != norbs.pop():
        raise ValueError('Single `onsite` matrix of shape ({0}, {0}) '
                         'provided but there are a different number of '
                         'orbitals per site in the system'.format(M.shape[0]))
    return M


class _LocalOperator:
    """Common part of Density / Current (kwant/operator.pyx:418-720)."""

    def __init__(self, syst, onsite, where, *, check_hermiticity=True,
                 sum=False):
        if getattr(syst, 'site_ranges', None) is None:
            raise ValueError('Number of orbitals not defined.')
        self.syst = syst
        self.onsite = _normalize_onsite(syst, onsite, check_hermiticity)
        self.check_hermiticity = check_hermiticity
        self.sum = sum
        self._site_ranges = np.asarray(syst.site_ranges, dtype=gint_dtype)
        self.where = where
        self._bound_params = None
        self._bound = False
        self._device = {}

    def bind(self, args=(), *, params=None):
        if args:
            raise TypeError("positional 'args' are not supported; use "
                            "'params'")
        q = self.__class__.__new__(self.__class__)
        q.__dict__.update(self.__dict__)
        q._bound_params = params
        q._bound = True
        q._device = {}
        return q

    def _params(self, args, params):
        if self._bound and (args or params):
            raise ValueError("Extra arguments are already bound to this "
                             "operator. You should call this operator "
                             "providing neither 'args' nor 'params'.")
        if args:
            raise TypeError("positional 'args' are not supported; use "
                            "'params'")
        return self._bound_params if self._bound else params

    def _tot_norbs(self):
        return int(self._site_ranges[-1, 2])

    def _lowered(self, params):
        return lower(self, params=params)

    def _device_op(self, params):
        from . import _lib
        key = ('op', repr(params))
        if key not in self._device:
            n = self._tot_norbs()
            ident = sp.identity(n, dtype=complex, format='csr')
            h = _lib.Handle(ident, 1.0, 0.0, _lib.PREC_FP64)
            self._device[key] = (h, _lib.Op(h, self._lowered(params)))
        return self._device[key][1]

    def __call__(self, bra, ket=None, args=(), *, params=None):
        """MAT_ELS on the device (kwant/operator.pyx:470-559)."""
        params = self._params(args, params)
        if bra is None:
            raise TypeError('bra must be an array')
        bra = np.asarray(bra, dtype=complex)
        same = ket is None or ket is bra
        ket = bra if ket is None else np.asarray(ket, dtype=complex)
        n = self._tot_norbs()
        if bra.shape != (n,):
            raise ValueError('bra vector is incorrect shape')
        if ket.shape != (n,):
            raise ValueError('ket vector is incorrect shape')
        res = self._device_op(params).apply(bra, ket)
        if self.check_hermiticity and same:
            res = res.real
        return res[0] if self.sum else res

    def act(self, ket, args=(), *, params=None):
        """ACT on the device (kwant/operator.pyx:561-606)."""
        from . import _lib
        params = self._params(args, params)
        if ket is None:
            raise TypeError('ket must be an array')
        ket = np.asarray(ket, dtype=complex)
        n = self._tot_norbs()
        if ket.shape != (n,):
            raise ValueError('ket vector is incorrect shape')
        key = ('act', repr(params))
        if key not in self._device:
            m = act_matrix(self, n, params)
            self._device[key] = _lib.Handle(m, 1.0, 0.0, _lib.PREC_FP64)
        return self._device[key].matvec(ket)

    def tocoo(self, args=(), *, params=None):
        params = self._params(args, params)
        return act_matrix(self, self._tot_norbs(), params).tocoo()


class Density(_LocalOperator):
    """kwant/operator.pyx:723-868."""

    def __init__(self, syst, onsite=1, where=None, *, check_hermiticity=True,
                 sum=False):
        where = _normalize_site_where(syst, where)
        super().__init__(syst, onsite, where,
                         check_hermiticity=check_hermiticity, sum=sum)


class Source(_LocalOperator):
    """kwant/operator.pyx:1003-1126: the source of a density M, the
    per-site tensor i [(H_aa)^dagger M_a - M_a H_aa]."""

    def __init__(self, syst, onsite=1, where=None, *, check_hermiticity=True,
                 sum=False):
        where = _normalize_site_where(syst, where)
        super().__init__(syst, onsite, where,
                         check_hermiticity=check_hermiticity, sum=sum)


class Current(_LocalOperator):
    """kwant/operator.pyx:871-1000."""

    def __init__(self, syst, onsite=1, where=None, *, check_hermiticity=True,
                 sum=False):
        where = _normalize_hopping_where(syst, where)
        super().__init__(syst, onsite, where,
                         check_hermiticity=check_hermiticity, sum=sum)


# --------------------------------------------------------------------------
# Lowering of any supported operator
# --------------------------------------------------------------------------

def _eval_onsites(syst, onsite, sites, params):
    """Per-site onsite matrices for a callable / mapping onsite."""
    out = []
    for s in sites:
        s = int(s)
        if isinstance(onsite, collections.abc.Mapping):
            M = onsite[syst.sites[s].family]
        else:
            site = syst.sites[s] if hasattr(syst, 'sites') else s
            if params:
                import inspect
                names = list(inspect.signature(onsite).parameters)[1:]
                M = onsite(site, *[params[n] for n in names])
            else:
                M = onsite(site)
        M = np.asarray(M, complex)
        out.append(M.reshape(1, 1) if M.ndim == 0 else M)
    return out


def _hop_blocks(syst, hops, params):
    if hasattr(syst, 'hamiltonian_blocks'):
        return syst.hamiltonian_blocks(hops)
    out = []
    for a, b in hops:
        m = syst.hamiltonian(int(a), int(b), params=params)
        m = np.asarray(m, complex)
        out.append(m.reshape(1, 1) if m.ndim == 0 else m)
    return out


def _blocks_from_bsm(bsm):
    """Matrices of a reference BlockSparseMatrix (kwant/operator.pyx:324-407)."""
    data = np.asarray(bsm.data)
    offs = np.asarray(bsm.data_offsets)
    shapes = np.asarray(bsm.block_shapes)
    return [data[o:o + r * c].reshape(r, c)
            for o, (r, c) in zip(offs, shapes)]


def _operator_info(op, params=None):
    """Kind, where, onsite matrices and hopping blocks of a Density or
    Current, from this module or from the reference kwant.operator."""
    name = type(op).__name__
    if name not in ('Density', 'Current', 'Source'):
        raise NotImplementedError(
            'operator %r cannot be lowered to the device' % (op,))
    where = np.asarray(op.where, dtype=np.int64)
    site_ranges = np.asarray(op._site_ranges, dtype=np.int64)
    onsite = op.onsite
    ours = isinstance(op, _LocalOperator)
    if ours:
        params = op._bound_params if op._bound else params
    kind = 'current' if name == 'Current' else 'density'
    if callable(onsite) or isinstance(onsite, collections.abc.Mapping):
        bound = getattr(op, '_bound_onsite', None) if not ours else None
        if bound is not None:
            mats = _blocks_from_bsm(bound)
        else:
            mats = _eval_onsites(op.syst, onsite, where[:, 0], params)
    else:
        mats = np.asarray(onsite, complex)
    if name == 'Source':
        # Source MAT_ELS / ACT (kwant/operator.pyx:1062-1126) is a density
        # with the per-site matrix Q_a = i (H_aa^dagger M_a - M_a H_aa)
        sites = where.reshape(-1)
        bound = getattr(op, '_bound_hamiltonian', None) if not ours else None
        if bound is not None:
            H_aa = _blocks_from_bsm(bound)
        else:
            H_aa = _hop_blocks(op.syst, np.stack([sites, sites], axis=1),
                               params)
        _, norbs = _site_orbitals(site_ranges, sites)
        Ms = _blocks_for(mats if isinstance(mats, list) else mats, norbs)
        mats = []
        for w in range(len(sites)):
            n = int(norbs[w])
            H = np.asarray(H_aa[w], complex).reshape(n, n)
            M = Ms[w]
            mats.append(1j * (H.conj().T @ M - M @ H))
    info = dict(kind=kind, where=where if kind == 'current'
                else where.reshape(-1), site_ranges=site_ranges,
                onsite=mats, sum=bool(op.sum),
                check_hermiticity=bool(op.check_hermiticity))
    if kind == 'current':
        bound = getattr(op, '_bound_hamiltonian', None) if not ours else None
        if bound is not None:
            info['hop_blocks'] = _blocks_from_bsm(bound)
        else:
            info['hop_blocks'] = _hop_blocks(op.syst, where, params)
    return info


def lower(op, params=None):
    """Lower a Density / Current (ours or the reference's, bound or not) to
    the device term form."""
    info = _operator_info(op, params)
    if info['kind'] == 'density':
        return lower_density(info['site_ranges'], info['where'],
                             info['onsite'], info['sum'],
                             info['check_hermiticity'])
    return lower_current(info['site_ranges'], info['where'],
                         info['hop_blocks'], info['onsite'], info['sum'],
                         info['check_hermiticity'])
