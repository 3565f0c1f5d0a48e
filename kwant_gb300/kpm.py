"""Kernel polynomial method on a GB300: drop-in for ``kwant.kpm``.

Same public API as kwant/kpm.py (``SpectralDensity``, ``Correlator``,
``conductivity``, ``RandomVectors``, ``LocalVectors``, ``jackson_kernel``,
``lorentz_kernel``, ``fermi_distribution``; kwant/kpm.py:32-34) with the hot
path on the device:

* the Chebyshev recursion of all vectors of a call runs as one batched,
  fused sparse x multi-vector pass per step (``csrc/kpm_core.cu``), with the
  moment dot products (DOS) or the operator (Density / Current / matrix,
  ``csrc/kpm_ops.cu``) evaluated in the same step sequence;
* the mean over vectors, the 1/a scale, the Jackson / Lorentz kernel and the
  DCT-III reconstruction run on the device (``csrc/kpm_recon.cu``);
* spectral bounds come from a device Lanczos (``csrc/kpm_lanczos.cu``), or
  from ARPACK driving device matvecs (``bounds_method='arpack'``, which
  reproduces the reference's bounds);
* the correlator's two recursions and its moments-matrix contraction run on
  the device (``csrc/kpm_correlator.cu``, ``csrc/kpm_gemm*.cu``).

Extra keyword-only arguments: ``precision`` ('fp64': complex128 recursion in
the reference's CSR order, with fused multiply-adds; 'mixed': complex64 recursion, which for
the DOS keeps a bfloat16 correction next to every complex64 element and
steps with error-free FP32 transformations, so the per-orbital DOS stays
within ~1e-6 of FP64 at every Chebyshev node; 'single': the plain complex64
recursion, a third fewer bytes per step, up to ~1e-4 off at the outermost
nodes) and ``bounds_method``.

Host code keeps the reference's semantics for everything that is not
arithmetic on the vectors: argument checks and error messages, the random
vector stream (``_v0`` first, then one block per vector from the same
MT19937 stream), ``real_if_close``, resume bookkeeping and the cheap
post-processing (``__call__`` at arbitrary energies, ``integrate``,
``Correlator.__call__``).
"""

import itertools
import math
from collections.abc import Iterable

import numpy as np
from scipy.integrate import simpson
from scipy.sparse import coo_matrix, csr_matrix
from scipy.sparse.linalg import LinearOperator, eigsh

from . import _lib
from . import operator as _operator

__all__ = ['SpectralDensity', 'Correlator', 'conductivity',
           'RandomVectors', 'LocalVectors', 'jackson_kernel', 'lorentz_kernel',
           'fermi_distribution']

SAMPLING = 2  # kwant/kpm.py:36

_PRECISIONS = {'fp64': _lib.PREC_FP64, 'double': _lib.PREC_FP64,
               'mixed': _lib.PREC_MIXED, 'single': _lib.PREC_SINGLE}


# --------------------------------------------------------------------------
# helpers mirroring the reference
# --------------------------------------------------------------------------

def ensure_rng(rng=None):
    """kwant/_common.py:115-135."""
    if rng is None:
        return np.random.mtrand._rand
    if isinstance(rng, (int, np.integer)):
        return np.random.RandomState(rng)
    if all(hasattr(rng, attr) for attr in ('random_sample', 'randn',
                                           'randint', 'choice')):
        return rng
    raise ValueError("Expecting a seed or an object that offers the "
                     "numpy.random.RandomState interface.")


def _is_system(obj):
    """A Kwant-like finite system (kwant.system.System or LatticeSystem)."""
    return hasattr(obj, 'hamiltonian_submatrix') and hasattr(obj, 'graph')


def _is_local_operator(obj):
    return type(obj).__name__ in ('Density', 'Current', 'Source') and \
        hasattr(obj, 'where') and hasattr(obj, 'bind')


def _kernel_id(kernel):
    """Device id of a known kernel callable, else None."""
    name = getattr(kernel, '__name__', None)
    mod = getattr(kernel, '__module__', '') or ''
    if name == 'jackson_kernel' and ('kpm' in mod):
        return _lib.KERNEL_JACKSON
    if name == 'lorentz_kernel' and ('kpm' in mod):
        return _lib.KERNEL_LORENTZ
    return None


def _precision(precision):
    try:
        return _PRECISIONS[precision]
    except KeyError:
        raise ValueError("precision must be one of %s"
                         % sorted(_PRECISIONS)) from None


def _reorder_default(reorder, precision):
    if reorder is None:
        return precision in (_lib.PREC_MIXED, _lib.PREC_SINGLE)
    return bool(reorder)


def _simpson_weights(x):
    """Weights w with sum(w * y) = scipy.integrate.simpson(y, x=x), the
    quadrature of Correlator.__call__ (kwant/kpm.py:627): the composite
    Simpson rule for irregularly spaced points (parabola through each pair
    of intervals), and for an even number of points Simpson on all but the
    last interval plus Cartwright's correction for it (the form scipy uses
    since 1.11).  Simpson is linear in y, so the weights depend on x only."""
    x = np.asarray(x, dtype=float)
    n = x.size
    w = np.zeros(n)
    if n < 2:
        return w
    h = np.diff(x)
    if n == 2:
        return np.full(2, 0.5 * h[0])
    stop = n - 2 if n % 2 else n - 3          # triples (i, i+1, i+2)
    for i in range(0, stop, 2):
        h0, h1 = h[i], h[i + 1]
        hs, hp = h0 + h1, h0 * h1
        w[i] += hs / 6.0 * (2.0 - h1 / h0)
        w[i + 1] += hs / 6.0 * (hs * hs / hp)
        w[i + 2] += hs / 6.0 * (2.0 - h0 / h1)
    if n % 2 == 0:
        h0, h1 = h[-2], h[-1]
        w[-1] += (2 * h1 ** 2 + 3 * h0 * h1) / (6 * (h1 + h0))
        w[-2] += (h1 ** 2 + 3.0 * h0 * h1) / (6 * h0)
        w[-3] -= h1 ** 3 / (6 * h0 * (h0 + h1))
    return w


def _chebyshev_nodes(n_sampling):
    """kwant/kpm.py:1190-1194."""
    raw, step = np.linspace(np.pi, 0, n_sampling, endpoint=False,
                            retstep=True)
    return np.cos(raw + step / 2)


def jackson_kernel(moments):
    """Convolutes ``moments`` with the Jackson kernel (kwant/kpm.py:1106-1123,
    Rev. Mod. Phys. 78, 275, Eq. 71).  Host version for user code; the
    density reconstruction applies the same weights on the device."""
    n_moments = len(moments)
    m = np.arange(n_moments)
    kernel_array = ((n_moments - m + 1) *
                    np.cos(np.pi * m / (n_moments + 1)) +
                    np.sin(np.pi * m / (n_moments + 1)) /
                    np.tan(np.pi / (n_moments + 1)))
    kernel_array /= n_moments + 1
    return np.transpose(np.transpose(moments) * kernel_array)


def lorentz_kernel(moments, l=4):
    """Convolutes ``moments`` with the Lorentz kernel
    (kwant/kpm.py:1126-1142)."""
    n_moments = len(moments)
    m = np.arange(n_moments)
    kernel_array = np.sinh(l * (1 - m / n_moments)) / np.sinh(l)
    return np.transpose(np.transpose(moments) * kernel_array)


def fermi_distribution(energy, mu, temperature):
    """kwant/kpm.py:990-1009."""
    if temperature < 0:
        raise ValueError("temperature must be non-negative")
    elif temperature == 0:
        return np.array(np.less(energy - mu, 0), dtype=float)
    else:
        return 1 / (1 + np.exp((energy - mu) / temperature))


def _rescale_ab(lmin, lmax, eps):
    """kwant/kpm.py:1174-1180."""
    tol = eps / 2
    a = np.abs(lmax - lmin) / (2. - eps)
    b = (lmax + lmin) / 2.
    if lmax - lmin <= abs(lmax + lmin) * tol / 2:
        raise ValueError(
            'The Hamiltonian has a single eigenvalue, it is not possible to '
            'obtain a spectral density.')
    return a, b


def spectral_bounds(hamiltonian, eps=0.05, v0=None, method='lanczos'):
    """Lowest and highest eigenvalue of ``hamiltonian`` (the two eigsh calls
    of kwant/kpm.py:1169-1172).  'lanczos': FP64 Lanczos on the device with
    Ritz-residual widening; 'arpack': scipy's ARPACK (tol = eps/2) with every
    matvec on the device, which reproduces the reference's bounds."""
    ham = csr_matrix(hamiltonian)
    n = ham.shape[0]
    if v0 is None:
        v0 = np.exp(2j * np.pi * np.random.RandomState(0).random_sample(n))
    tol = eps / 2
    if method == 'lanczos':
        lo, hi, _ = _lib.bounds(ham, v0, tol, max_iter=max(50, min(n, 3000)))
        return lo, hi
    if method == 'arpack':
        h = _lib.Handle(ham, 1.0, 0.0, _lib.PREC_FP64)
        op = LinearOperator(shape=ham.shape, matvec=h.matvec, dtype=complex)
        try:
            lmax = eigsh(op, k=1, which='LA', return_eigenvectors=False,
                         tol=tol, v0=v0)[0]
            lmin = eigsh(op, k=1, which='SA', return_eigenvectors=False,
                         tol=tol, v0=v0)[0]
        finally:
            h.close()
        return lmin, lmax
    raise ValueError("bounds_method must be 'lanczos' or 'arpack'")


class _RescaledHamiltonian(LinearOperator):
    """The reference's ``SpectralDensity.hamiltonian`` (kwant/kpm.py:1182-1185)
    with the matvec on the device."""

    def __init__(self, ham, a, b):
        self._ham = ham
        self._a, self._b = a, b
        self._dev = None
        super().__init__(dtype=complex, shape=ham.shape)

    def _matvec(self, v):
        if self._dev is None:
            self._dev = _lib.Handle(self._ham, 1.0, 0.0, _lib.PREC_FP64)
        v = np.asarray(v, complex).ravel()
        return (self._dev.matvec(v) - self._b * v) / self._a


# --------------------------------------------------------------------------
# vector factories (kwant/kpm.py:850-985)
# --------------------------------------------------------------------------

class _SequenceTail:
    """A sequence of vectors resumed after its first ``start`` elements:
    its length is the sequence's, its iteration starts at ``start``."""

    def __init__(self, seq, start):
        self.seq, self.start = seq, start

    def __len__(self):
        return len(self.seq)

    def __iter__(self):
        return itertools.islice(iter(self.seq), self.start, None)


class _VectorFactory:
    """kwant/kpm.py:850-929."""

    def __init__(self, vectors=None, num_vectors=None, accumulate=True):
        assert isinstance(vectors, Iterable)
        try:
            _len = len(vectors)
            if num_vectors is None:
                num_vectors = _len
        except TypeError:
            _len = np.inf
            if num_vectors is None:
                raise ValueError("'num_vectors' must be specified when "
                                 "'vectors' has no len() method.")
        self._max_vectors = _len
        self._iterator = iter(vectors)
        self.accumulate = accumulate
        self.saved_vectors = []
        self.num_vectors = 0
        self.add_vectors(num_vectors=num_vectors)
        self._last_idx = -np.inf
        self._last_vector = None

    def _fill_in_saved_vectors(self, index):
        if index < self._last_idx and not self.accumulate:
            raise ValueError("Cannot get previous values if 'accumulate' "
                             "is False")
        if index >= self.num_vectors:
            raise IndexError('Requested more vectors than available')
        self._last_idx = index
        if self.accumulate:
            if self.saved_vectors[index] is None:
                self.saved_vectors[index] = next(self._iterator)
        else:
            self._last_vector = next(self._iterator)

    def __getitem__(self, index):
        self._fill_in_saved_vectors(index)
        if self.accumulate:
            return self.saved_vectors[index]
        return self._last_vector

    def add_vectors(self, num_vectors=None):
        if num_vectors is None:
            raise ValueError("'num_vectors' must be specified.")
        else:
            if num_vectors <= 0 or num_vectors != int(num_vectors):
                raise ValueError("'num_vectors' must be a positive integer")
            elif self.num_vectors + num_vectors > self._max_vectors:
                raise ValueError("'num_vectors' is larger than available "
                                 "vectors")
        self.num_vectors += num_vectors
        if self.accumulate:
            self.saved_vectors.extend([None] * num_vectors)


def _normalize_orbs_where(syst, where):
    """kwant/kpm.py:1025-1039 (and _from_where_to_orbs, :1012-1022)."""
    if _is_system(syst):
        sr = np.asarray(syst.site_ranges, dtype=np.int64)
        tot_norbs = int(sr[-1, 2])
        where = _operator._normalize_site_where(syst, where)
        start, norbs = _operator._site_orbitals(sr, where.reshape(-1))
        orbs = []
        for s, n in zip(start, norbs):
            orbs.extend(range(s, s + n))
    else:
        try:
            tot_norbs = csr_matrix(syst).shape[0]
        except TypeError:
            raise TypeError("'syst' is neither a matrix "
                            "nor a Kwant system.")
        orbs = (range(tot_norbs) if where is None
                else np.asarray(where, int))
    return tot_norbs, orbs


_PHASE_POOL = None


def _host_pool():
    """Thread pool over the host's cores for numpy work that releases the
    GIL (complex exp, large copies)."""
    global _PHASE_POOL
    if _PHASE_POOL is None:
        import concurrent.futures
        import os
        _PHASE_POOL = concurrent.futures.ThreadPoolExecutor(
            max_workers=max(1, min(32, os.cpu_count() or 1)))
    return _PHASE_POOL


def _phases(u):
    """exp(2j * pi * u) elementwise, bit-identical to numpy's expression
    (the same ufuncs on each element), computed in chunks on the host's
    cores for long vectors (numpy's complex exp is single-threaded)."""
    n = u.shape[0]
    chunk = 1 << 18
    if n < 4 * chunk:
        return np.exp(2j * np.pi * u)
    out = np.empty(n, dtype=complex)

    def work(i):
        out[i:i + chunk] = np.exp(2j * np.pi * u[i:i + chunk])

    list(_host_pool().map(work, range(0, n, chunk)))
    return out


def _stack_vectors(vectors):
    """The vectors as the rows of one complex array (what np.array makes of
    them), copied on the host's cores when they are large."""
    vs = [np.asarray(v, complex) for v in vectors]
    n = vs[0].shape[0] if vs and vs[0].ndim == 1 else -1
    if n < (1 << 20) or any(v.ndim != 1 or v.shape[0] != n for v in vs):
        return np.array(vs)
    out = np.empty((len(vs), n), dtype=complex)

    def work(i):
        out[i] = vs[i]

    list(_host_pool().map(work, range(len(vs))))
    return out


def RandomVectors(syst, where=None, rng=None):
    """Random-phase vectors exp(2 pi i u) on the orbitals of ``where``
    (kwant/kpm.py:932-951): the same stream and values as the reference."""
    rng = ensure_rng(rng)
    tot_norbs, orbs = _normalize_orbs_where(syst, where)
    idx = np.asarray(orbs, dtype=np.intp)
    full = idx.shape[0] == tot_norbs and np.array_equal(
        idx, np.arange(tot_norbs))
    while True:
        phases = _phases(rng.random_sample(idx.shape[0]))
        if full:
            yield phases
        else:
            vector = np.zeros(tot_norbs, dtype=complex)
            vector[idx] = phases
            yield vector


class LocalVectors:
    """Unit vectors on the orbitals of ``where`` (kwant/kpm.py:954-985)."""

    def __init__(self, syst, where=None, *args):
        self.tot_norbs, self.orbs = _normalize_orbs_where(syst, where)
        self._idx = 0

    def __len__(self):
        return len(self.orbs)

    def __iter__(self):
        return self

    def __next__(self):
        if self._idx < len(self):
            vector = np.zeros(self.tot_norbs)
            vector[self.orbs[self._idx]] = 1
            self._idx = self._idx + 1
            return vector
        raise StopIteration('Too many vectors requested from this generator')


# --------------------------------------------------------------------------
# SpectralDensity
# --------------------------------------------------------------------------

class _Batch:
    """Vectors [r0, r0 + R) of a SpectralDensity with their device state."""

    def __init__(self, r0, block):
        self.r0 = r0
        self.block = block


class SpectralDensity:
    r"""Spectral density of an operator by the kernel polynomial method.

    Drop-in for ``kwant.kpm.SpectralDensity`` (kwant/kpm.py:39-490); see the
    module docstring for what runs on the device.  ``energies``,
    ``densities``, ``num_moments``, ``num_vectors``, ``bounds``, ``eps``,
    ``kernel``, ``mean``, ``__call__``, ``integrate``, ``add_moments`` and
    ``add_vectors`` behave as in the reference.

    Extra keyword-only parameters
    -----------------------------
    precision : 'fp64' (default), 'mixed' or 'single'
    bounds_method : 'lanczos' (default) or 'arpack'
    reorder : bool, optional
        Store the Hamiltonian in a bandwidth-reducing (RCM) order on the
        device; default: on for 'mixed' and 'single', off for 'fp64'.  Results are
        invariant up to rounding.
    """

    def __init__(self, hamiltonian, params=None, operator=None,
                 num_vectors=10, num_moments=None, energy_resolution=None,
                 vector_factory=None, bounds=None, eps=0.05, rng=None,
                 kernel=None, mean=True, accumulate_vectors=True, *,
                 precision='fp64', bounds_method='lanczos', reorder=None):

        if num_moments and energy_resolution:
            raise TypeError("either 'num_moments' or 'energy_resolution' "
                            "must be provided.")
        self.eps = eps
        self._precision = _precision(precision)

        hamiltonian = self._bind(hamiltonian, params, operator)

        self.mean = mean
        rng = ensure_rng(rng)
        self._rng = rng if vector_factory is None else None
        self._reorder = _reorder_default(reorder, self._precision)
        self._v0 = np.exp(2j * np.pi * rng.random_sample(hamiltonian.shape[0]))

        if eps <= 0:
            raise ValueError("'eps' must be positive")

        if bounds:
            lmin, lmax = bounds
        else:
            lmin, lmax = spectral_bounds(hamiltonian, eps, self._v0,
                                         bounds_method)
        self._a, self._b = _rescale_ab(lmin, lmax, eps)
        self._ham_csr = hamiltonian
        self.hamiltonian = _RescaledHamiltonian(hamiltonian, self._a, self._b)
        self.bounds = (self._b - self._a, self._b + self._a)

        if energy_resolution:
            num_moments = math.ceil((1.6 * self._a) / energy_resolution)
        elif num_moments is None:
            num_moments = 100
        if num_moments <= 0 or num_moments != int(num_moments):
            raise ValueError("'num_moments' must be a positive integer")
        num_moments = int(num_moments)
        if num_moments < 2:
            raise ValueError("'num_moments' must be at least 2")

        if vector_factory is None:
            self._vector_factory = _VectorFactory(
                RandomVectors(hamiltonian, rng=rng),
                num_vectors=num_vectors, accumulate=accumulate_vectors)
        else:
            if not isinstance(vector_factory, Iterable):
                raise TypeError('vector_factory must be iterable')
            try:
                len(vector_factory)
            except TypeError:
                if num_vectors is None:
                    raise ValueError('num_vectors must be provided if'
                                     'vector_factory has no length.')
            self._vector_factory = _VectorFactory(
                vector_factory, num_vectors=num_vectors,
                accumulate=accumulate_vectors)
        num_vectors = self._vector_factory.num_vectors

        self._handle = _lib.Handle(_lib.Csr(hamiltonian), self._a, self._b,
                                   self._precision, reorder=self._reorder)
        self._op = None if self._lowered is None else \
            _lib.Op(self._handle, self._lowered)
        self._batches = []
        self._moments_arr = None   # (R, M) or (R, M, W) complex128

        self.num_moments = 0
        self._update_moments_list(num_moments, num_vectors)
        self.num_moments = num_moments

        self.kernel = kernel if kernel is not None else jackson_kernel
        self._reconstruct()

    def _bind(self, hamiltonian, params, operator):
        """Hamiltonian as CSR and the operator lowered to the device term
        form (kwant/kpm.py:172-198)."""
        if _is_system(hamiltonian):
            hamiltonian = hamiltonian.hamiltonian_submatrix(params=params,
                                                            sparse=True)
        try:
            hamiltonian = csr_matrix(hamiltonian)
        except Exception:
            raise ValueError("'hamiltonian' is neither a matrix "
                             "nor a Kwant system.")
        if hamiltonian.ndim != 2 or hamiltonian.shape[0] != \
                hamiltonian.shape[1]:
            raise ValueError("'hamiltonian' is neither a matrix "
                             "nor a Kwant system.")

        # operator: lowered to the device term form (kwant/kpm.py:187-198)
        if operator is None:
            self.operator = None
            self._lowered = None
        elif _is_local_operator(operator):
            self.operator = operator.bind(params=params)
            self._lowered = _operator.lower(self.operator, params=params)
        elif callable(operator):
            raise NotImplementedError(
                'an arbitrary Python callable operator cannot run on the '
                'device; pass a kwant Density/Current operator or a matrix')
        elif hasattr(operator, 'dot'):
            operator = csr_matrix(operator)
            self.operator = operator
            self._lowered = _operator.lower_matrix(operator)
        else:
            raise ValueError("Parameter 'operator' has no '.dot' "
                             "attribute and is not callable.")
        return hamiltonian

    # -- public properties -------------------------------------------------
    @property
    def energies(self):
        return (self._a * _chebyshev_nodes(SAMPLING * self.num_moments)
                + self._b)

    @property
    def num_vectors(self):
        return 0 if self._moments_arr is None else self._moments_arr.shape[0]

    @property
    def _moments_list(self):
        """Per-vector moments, as the reference stores them
        (kwant/kpm.py:486-490)."""
        if self._moments_arr is None:
            return []
        arr = self._moments_arr
        if self._lowered is None or self._lowered.scalar:
            arr = arr[..., 0]
        return list(arr)

    @property
    def _last_two_alphas(self):
        """(alpha_{n-1}, alpha_n) of every vector, read from the device."""
        out = []
        for batch in self._batches:
            prev, cur = batch.block.state()
            out.extend(zip(prev, cur))
        return out

    # -- moments -------------------------------------------------------------
    def _block_moments(self, block, m_start, m_end):
        if self._op is None:
            # divergence is reported by _check_divergence (a warning, as
            # the reference returns its moments unchecked)
            return block.dos_moments(m_start, m_end, diverged='return')
        return block.op_moments(self._op, m_start, m_end)

    def _update_moments_list(self, n_moments, num_vectors):
        """kwant/kpm.py:390-490 on the device."""
        have = self.num_vectors
        if have == num_vectors:
            new_vectors = 0
        elif have < num_vectors:
            new_vectors = num_vectors - have
        else:
            raise ValueError('Cannot decrease number of vectors')

        if n_moments == self.num_moments:
            new_moments = 0
            if new_vectors == 0:
                return
        else:
            if not self._vector_factory.accumulate and self.num_moments:
                raise ValueError("Cannot increase the number of moments if "
                                 "'accumulate_vectors' is 'False'.")
            new_moments = n_moments - self.num_moments
            if new_moments < 0:
                raise ValueError('Cannot decrease number of moments')
            if new_vectors != 0 and self.num_moments:
                raise ValueError("Only 'num_moments' *or* 'num_vectors' "
                                 "may be updated at a time.")

        if new_vectors:
            vecs = _stack_vectors(self._vector_factory[r]
                                  for r in range(have, num_vectors))
            if vecs.ndim != 2 or vecs.shape[1] != self._ham_csr.shape[0]:
                raise ValueError('vectors must have the length of the '
                                 'Hamiltonian')
            keep = self._vector_factory.accumulate or self._op is not None
            block = _lib.Block(self._handle, vecs, keep_a0=keep)
            mom = self._block_moments(block, 0, n_moments)
            if self._op is None:
                mom = mom[:, :, None]
            self._moments_arr = mom if self._moments_arr is None else \
                np.concatenate([self._moments_arr, mom], axis=0)
            if self._vector_factory.accumulate:
                self._batches.append(_Batch(have, block))
            else:
                block.close()
        elif new_moments:
            parts = []
            for batch in self._batches:
                mom = self._block_moments(batch.block, self.num_moments,
                                          n_moments)
                if self._op is None:
                    mom = mom[:, :, None]
                parts.append(mom)
            self._moments_arr = np.concatenate(
                [self._moments_arr, np.concatenate(parts, axis=0)], axis=1)

    def _moments(self):
        """kwant/kpm.py:378-388 (host copy of the reduced moments)."""
        moments = np.real_if_close(self._moments_list)
        moments = np.swapaxes(moments, 0, 1)
        if self.mean:
            moments = np.mean(moments, axis=1)
        moments /= self._a
        return self.kernel(moments)

    def _check_divergence(self):
        """Failure detection for spectral bounds that are too tight: the DOS
        moments of a vector obey |mu_n| <= mu_0 when the rescaled spectrum
        lies in [-1, 1] (|T_n| <= 1 there); a bound that leaves eigenvalues
        outside makes T_n grow exponentially.  The reference does not check
        this; here it is reported with a warning (results are returned
        unchanged, as the reference would)."""
        if self._lowered is not None or self._moments_arr is None:
            return
        mom = self._moments_arr[:, :, 0]
        mu0 = np.abs(mom[:, :1].real)
        if np.any(np.abs(mom) > 1.01 * mu0 + 1e-300):
            import warnings
            warnings.warn('Chebyshev moments exceed mu_0: the spectral bounds '
                          '%r do not enclose the spectrum; the recursion '
                          'diverged' % (self.bounds,), RuntimeWarning,
                          stacklevel=3)

    def _reconstruct(self):
        """Mean, 1/a, kernel and DCT on the device (kwant/kpm.py:251-252)."""
        self._check_divergence()
        arr = self._moments_arr                      # (R, M, W)
        R, M, W = arr.shape
        is_real = bool(np.all(np.abs(arr.imag) <
                              100 * np.finfo(np.float64).eps))
        nodes = _chebyshev_nodes(SAMPLING * M)
        kid = _kernel_id(self.kernel)
        if kid is not None:
            gam, rho = _lib.reconstruct(arr, self.mean, is_real, self._a, kid,
                                        4.0, nodes)
        else:
            # user kernel: runs on the host (user code); DCT on the device
            mom = self._moments()
            mom = np.asarray(mom)
            flat = mom.reshape(M, -1)
            gam, rho = _lib.reconstruct(
                np.ascontiguousarray(flat[None, :, :]), True,
                not np.iscomplexobj(flat), 1.0, _lib.KERNEL_NONE, 4.0, nodes)
        scalar = self._lowered is None or self._lowered.scalar
        if self.mean:
            shape = (2 * M,) if scalar else (2 * M, W)
        else:
            shape = (2 * M, R) if scalar else (2 * M, R, W)
        if is_real:
            gam, rho = gam.real, rho.real
        self._gammas = gam.reshape(shape)
        self.densities = rho.reshape(shape)

    # -- public methods ------------------------------------------------------
    def __call__(self, energy=None):
        """kwant/kpm.py:263-295."""
        if energy is None:
            return self.energies, self.densities
        energy = np.asarray(energy)
        e = (energy - self._b) / self._a
        g_e = (np.pi * np.sqrt(1 - e) * np.sqrt(1 + e))
        moments = self._moments()
        moments[1:] = 2 * moments[1:]
        # the chebval sum runs on the device, with numpy's arithmetic
        vals = _lib.chebval(e, moments)
        if not np.iscomplexobj(moments):
            vals = vals.real
        return np.transpose(vals / g_e)

    def integrate(self, distribution_function=None):
        """kwant/kpm.py:297-316: the Gauss-Chebyshev sum
        a / (2M) * sum_k gamma_k f(E_k), summed on the device (the
        distribution function, a Python callable, is evaluated on the
        host at the 2M energies)."""
        factor = self._a / (2 * self.num_moments)
        gam = np.asarray(self._gammas)
        vals = gam.reshape(gam.shape[0], -1)
        n = vals.shape[0]
        if distribution_function is None:
            d = np.ones(n)
        else:
            d = np.asarray(distribution_function(self.energies))
            d = np.broadcast_to(d, (n,))
        out = _lib.fermi_sums(self.energies, factor * d.real, vals)[0]
        if np.iscomplexobj(d):
            out = out + 1j * _lib.fermi_sums(self.energies, factor * d.imag,
                                             vals)[0]
        if not (np.iscomplexobj(gam) or np.iscomplexobj(d)):
            out = out.real
        return out[0] if gam.ndim == 1 else out.reshape(gam.shape[1:])

    def integrate_sweep(self, mu=0, temperature=0):
        """``integrate(lambda E: fermi_distribution(E, mu, T))`` for a
        whole grid of (mu, temperature) points in one device launch (no
        reference counterpart; the reference evaluates one distribution
        per call, kwant/kpm.py:297-316): mu and temperature broadcast
        against each other; the result has their broadcast shape (plus the
        operator's output shape)."""
        mu, temperature = np.broadcast_arrays(np.asarray(mu, float),
                                              np.asarray(temperature, float))
        if np.any(temperature < 0):
            raise ValueError("temperature must be non-negative")
        factor = self._a / (2 * self.num_moments)
        gam = np.asarray(self._gammas)
        vals = gam.reshape(gam.shape[0], -1)
        w = np.full(vals.shape[0], factor)
        out = _lib.fermi_sums(self.energies, w, vals, mu.ravel(),
                              temperature.ravel())
        if not np.iscomplexobj(gam):
            out = out.real
        return out.reshape(mu.shape + gam.shape[1:])

    def add_moments(self, num_moments=None, *, energy_resolution=None):
        """kwant/kpm.py:318-358."""
        if not ((num_moments is None) ^ (energy_resolution is None)):
            raise TypeError("either 'num_moments' or 'energy_resolution' "
                            "must be provided.")
        if energy_resolution:
            if energy_resolution <= 0:
                raise ValueError("'energy_resolution' must be positive")
            present_resolution = self._a * 1.6 / self.num_moments
            if present_resolution < energy_resolution:
                raise ValueError('Energy resolution is already smaller '
                                 'than the requested resolution')
            num_moments = math.ceil((1.6 * self._a) / energy_resolution)
        if (num_moments is None or num_moments <= 0
                or num_moments != int(num_moments)):
            raise ValueError("'num_moments' must be a positive integer")
        self._update_moments_list(self.num_moments + int(num_moments),
                                  self.num_vectors)
        self.num_moments += int(num_moments)
        self._reconstruct()

    # -- checkpoints (no reference counterpart) ------------------------------
    def save(self, file):
        """Write a checkpoint (numpy .npz) from which ``load`` resumes the
        recursion exactly: the moments, the state the reference keeps in
        memory (``_last_two_alphas`` and the per-vector mu_0, mu_1 of the
        DOS doubling, kwant/kpm.py:486-490), the starting vectors, the
        rescaling, the settings and the random-vector stream's state."""
        if not self._vector_factory.accumulate:
            raise ValueError("a checkpoint needs accumulate_vectors=True "
                             "(the recursion state of every vector)")
        kname = {jackson_kernel: 'jackson', lorentz_kernel: 'lorentz'}.get(
            self.kernel, '')
        d = {'version': 1, 'a': self._a, 'b': self._b, 'eps': self.eps,
             'n': self._ham_csr.shape[0], 'num_moments': self.num_moments,
             'mean': self.mean, 'precision': self._precision,
             'reorder': self._reorder, 'kernel': kname,
             'moments': self._moments_arr, 'num_blocks': len(self._batches)}
        if self._rng is not None and hasattr(self._rng, 'get_state'):
            _, keys, pos, has_gauss, gauss = self._rng.get_state()
            d.update(rng_keys=keys, rng_pos=pos, rng_has_gauss=has_gauss,
                     rng_gauss=gauss)
        saved = self._vector_factory.saved_vectors
        for k, batch in enumerate(self._batches):
            steps, mode, mu01, prev, cur = batch.block.checkpoint()
            R = batch.block.R
            d['b%d_r0' % k] = batch.r0
            d['b%d_a0' % k] = np.array([saved[r] for r in
                                        range(batch.r0, batch.r0 + R)],
                                       dtype=complex)
            d['b%d_steps' % k] = steps
            d['b%d_mode' % k] = mode
            d['b%d_mu01' % k] = mu01
            if steps > 0:
                d['b%d_prev' % k] = prev
                d['b%d_cur' % k] = cur
        np.savez(file, **d)

    @classmethod
    def load(cls, file, hamiltonian, params=None, operator=None, *,
             vector_factory=None, kernel=None):
        """A SpectralDensity resumed from ``save``'s checkpoint, on the same
        ``hamiltonian`` (and ``operator``, ``params``).  ``add_moments``
        continues the saved recursion; ``add_vectors`` continues the saved
        random-vector stream, or draws from ``vector_factory`` when the
        vectors were user-supplied: a sequence (with ``len()``) is taken to
        be the same vectors as before, and its first ``num_vectors`` (the
        saved ones) are skipped; an iterator without ``len()`` must yield
        only the vectors that come after the checkpoint.  ``kernel`` is
        needed when a custom kernel was used."""
        z = np.load(file, allow_pickle=False)
        if int(z['version']) != 1:
            raise ValueError('unknown checkpoint version')
        self = cls.__new__(cls)
        self.eps = float(z['eps'])
        self._precision = int(z['precision'])
        hamiltonian = self._bind(hamiltonian, params, operator)
        if hamiltonian.shape[0] != int(z['n']):
            raise ValueError('the checkpoint was written for a Hamiltonian '
                             'of size %d' % int(z['n']))
        self.mean = bool(z['mean'])
        self._a, self._b = float(z['a']), float(z['b'])
        self._v0 = None
        self._ham_csr = hamiltonian
        self.hamiltonian = _RescaledHamiltonian(hamiltonian, self._a, self._b)
        self.bounds = (self._b - self._a, self._b + self._a)
        self._reorder = bool(z['reorder'])
        nblk = int(z['num_blocks'])
        a0s = [z['b%d_a0' % k] for k in range(nblk)]
        nvec = sum(len(a) for a in a0s)
        self._rng = None
        if vector_factory is not None:
            try:
                len(vector_factory)
                source = _SequenceTail(vector_factory, nvec)
            except TypeError:
                source = vector_factory
        elif 'rng_keys' in z.files:
            rng = np.random.RandomState()
            rng.set_state(('MT19937', z['rng_keys'], int(z['rng_pos']),
                           int(z['rng_has_gauss']), float(z['rng_gauss'])))
            self._rng = rng
            source = RandomVectors(hamiltonian, rng=rng)
        else:
            source = iter(())
        self._vector_factory = _VectorFactory(source, num_vectors=nvec,
                                              accumulate=True)
        for k, a0 in enumerate(a0s):
            r0 = int(z['b%d_r0' % k])
            for j, v in enumerate(a0):
                self._vector_factory.saved_vectors[r0 + j] = v
        self._handle = _lib.Handle(_lib.Csr(hamiltonian), self._a, self._b,
                                   self._precision, reorder=self._reorder)
        self._op = None if self._lowered is None else \
            _lib.Op(self._handle, self._lowered)
        self._batches = []
        for k, a0 in enumerate(a0s):
            block = _lib.Block(self._handle, a0, keep_a0=True)
            steps = int(z['b%d_steps' % k])
            block.restore(steps, int(z['b%d_mode' % k]), z['b%d_mu01' % k],
                          z['b%d_prev' % k] if steps else None,
                          z['b%d_cur' % k] if steps else None)
            self._batches.append(_Batch(int(z['b%d_r0' % k]), block))
        self._moments_arr = z['moments']
        self.num_moments = int(z['num_moments'])
        kname = str(z['kernel'])
        if kernel is not None:
            self.kernel = kernel
        elif kname == 'jackson':
            self.kernel = jackson_kernel
        elif kname == 'lorentz':
            self.kernel = lorentz_kernel
        else:
            raise ValueError('the checkpoint used a custom kernel; pass it '
                             'as kernel=')
        self._reconstruct()
        return self

    def add_vectors(self, num_vectors=None):
        """kwant/kpm.py:360-376."""
        self._vector_factory.add_vectors(num_vectors)
        num_vectors = self._vector_factory.num_vectors - self.num_vectors
        self._update_moments_list(self.num_moments,
                                  self.num_vectors + num_vectors)
        self._reconstruct()


# --------------------------------------------------------------------------
# Correlator / conductivity
# --------------------------------------------------------------------------

def _operator_matrix(op, params, n):
    """CSR matrix of an operator acting to the right (kwant/kpm.py:1088-1103):
    None -> identity, Density/Current -> its ACT map, matrix -> itself."""
    if op is None:
        from scipy.sparse import identity
        return identity(n, dtype=complex, format='csr')
    if _is_local_operator(op):
        if isinstance(op, _operator._LocalOperator):
            op = op.bind(params=params) if not op._bound else op
        return _operator.act_matrix(op, n, params)
    if callable(op) and not hasattr(op, 'dot'):
        raise NotImplementedError(
            'an arbitrary Python callable operator cannot run on the '
            'device; pass a kwant operator or a matrix')
    if hasattr(op, 'dot'):
        return csr_matrix(op)
    raise TypeError("The operators must have a '.dot' "
                    "attribute or must be callable.")


class Correlator:
    """Response of the correlation between two operators
    (kwant/kpm.py:493-760), with both Chebyshev recursions and the
    moments-matrix contraction on the device.

    Extra keyword-only arguments: ``precision`` ('fp64' | 'mixed'),
    ``bounds_method``, ``gemm`` ('auto' | 'fp64' | 'bf16x3' | 'fp16x3').
    'auto' is 'bf16x3' (BF16 hi+lo products on the tensor cores, FP32
    accumulation) in mixed precision and 'fp64' otherwise; 'fp16x3' runs
    the same tensor-core products on FP16 hi+lo parts (11 instead of 8
    significant bits each, the same time), about 60x closer to the exact
    contraction on sigma_xy, and raises KPMDiverged if a vector entry
    exceeds the FP16 range.
    """

    def __init__(self, hamiltonian, operator1=None, operator2=None,
                 **kwargs):
        params = kwargs.get('params')
        self.mean = kwargs.get('mean', True)
        self._accumulate = kwargs.get('accumulate_vectors', False)
        precision = kwargs.pop('precision', 'fp64')
        bounds_method = kwargs.pop('bounds_method', 'lanczos')
        gemm = kwargs.pop('gemm', 'auto')
        reorder = kwargs.pop('reorder', None)
        self._gemm = {'auto': 2, 'fp64': 0, 'bf16x3': 1,
                      'bf16x3-simt': 3, 'fp16x3': 4,
                      'fp16x3-simt': 5}[gemm]
        self._precision = _precision(precision)
        self._reorder = _reorder_default(reorder, self._precision)
        kwargs.pop('operator', None)
        if _is_system(hamiltonian):
            hamiltonian = hamiltonian.hamiltonian_submatrix(params=params,
                                                            sparse=True)
        try:
            hamiltonian = csr_matrix(hamiltonian)
        except Exception:
            raise ValueError("'hamiltonian' is neither a matrix "
                             "nor a Kwant system.")
        n = hamiltonian.shape[0]
        self._ham_csr = hamiltonian
        self._op1 = _operator_matrix(operator1, params, n)
        self._op2 = _operator_matrix(operator2, params, n)

        # the state of the first SpectralDensity of the reference
        # (kwant/kpm.py:570-575): rng stream, _v0, bounds, num_moments
        num_moments = kwargs.get('num_moments')
        energy_resolution = kwargs.get('energy_resolution')
        if num_moments and energy_resolution:
            raise TypeError("either 'num_moments' or 'energy_resolution' "
                            "must be provided.")
        eps = kwargs.get('eps', 0.05)
        self.eps = eps
        rng_arg = kwargs.get('rng')
        rng = ensure_rng(rng_arg)
        self._v0 = np.exp(2j * np.pi * rng.random_sample(n))
        if eps <= 0:
            raise ValueError("'eps' must be positive")
        bounds = kwargs.get('bounds')
        if bounds:
            lmin, lmax = bounds
        else:
            lmin, lmax = spectral_bounds(hamiltonian, eps, self._v0,
                                         bounds_method)
        self._a, self._b = _rescale_ab(lmin, lmax, eps)
        # second recursion: bounds that reproduce (a, b) (kwant/kpm.py:576-579)
        _a = self._a * (1 - eps / 2)
        self._a2, self._b2 = _rescale_ab(self._b - _a, self._b + _a, eps)
        if energy_resolution:
            num_moments = math.ceil((1.6 * self._a) / energy_resolution)
        elif num_moments is None:
            num_moments = 100
        if num_moments <= 0 or num_moments != int(num_moments):
            raise ValueError("'num_moments' must be a positive integer")
        self.num_moments = int(num_moments)

        vector_factory = kwargs.get('vector_factory')
        num_vectors = kwargs.get('num_vectors', 10)
        if vector_factory is None:
            self._vector_factory = _VectorFactory(
                RandomVectors(hamiltonian, rng=rng), num_vectors=num_vectors,
                accumulate=True)
        else:
            if not isinstance(vector_factory, Iterable):
                raise TypeError('vector_factory must be iterable')
            try:
                len(vector_factory)
            except TypeError:
                if num_vectors is None:
                    raise ValueError('num_vectors must be provided if'
                                     'vector_factory has no length.')
            self._vector_factory = _VectorFactory(
                vector_factory, num_vectors=num_vectors, accumulate=True)
        # the reference's second SpectralDensity draws its own _v0 from the
        # same rng argument (kwant/kpm.py:598-599, :201-203)
        ensure_rng(rng_arg).random_sample(n)

        kernel = kwargs.get('kernel')
        self.kernel = kernel if kernel is not None else jackson_kernel
        self._handle = _lib.Handle(_lib.Csr(hamiltonian), self._a, self._b,
                                   self._precision, reorder=self._reorder)
        self._compute()

    @property
    def num_vectors(self):
        return self._vector_factory.num_vectors

    @property
    def energies(self):
        return (self._a * _chebyshev_nodes(SAMPLING * self.num_moments)
                + self._b)

    def _vectors(self):
        return _stack_vectors(self._vector_factory[r]
                              for r in range(self._vector_factory.num_vectors))

    def _compute(self):
        vecs = self._vectors()
        mu = _lib.correlator_moments(
            self._handle, self._a2, self._b2, self._op1, self._op2, vecs,
            self.num_moments, gemm=self._gemm, per_vector=not self.mean)
        self.moments_matrix = mu
        self._build_integral_factor()

    def _build_integral_factor(self):
        """kwant/kpm.py:720-760 on the device."""
        n_moments = self.num_moments
        g_kernel = self.kernel(np.ones(n_moments))
        g_kernel = np.asarray(g_kernel, dtype=float)
        g_kernel[0] /= 2
        nodes = (self.energies - self._b) / self._a
        if self.mean:
            self._integral_factor = _lib.integral_factor(
                self.moments_matrix, g_kernel, nodes)
        else:
            self._integral_factor = np.array(
                [_lib.integral_factor(m, g_kernel, nodes)
                 for m in self.moments_matrix]).T

    def __call__(self, mu=0, temperature=0):
        """kwant/kpm.py:608-630: prefactor * Simpson over the rescaled
        nodes of f(E; mu, T) / (1 - e^2)^2 * factor(e), summed on the
        device."""
        if temperature < 0:
            raise ValueError("temperature must be non-negative")
        return self.sweep(mu, temperature)[()]

    def sweep(self, mu=0, temperature=0):
        """``self(mu, temperature)`` over a grid in one device launch:
        ``mu`` and ``temperature`` broadcast against each other and the
        result has their broadcast shape (no reference counterpart: the
        reference evaluates one (mu, temperature) per call,
        kwant/kpm.py:608-630).  The Simpson weights of the rescaled nodes,
        the (1 - e^2)^-2 factor and the prefactor 2 * 4^2 / (2a)^2 are
        folded into one weight per node on the host; the Fermi function
        and the sums over nodes run on the device."""
        mu, temperature = np.broadcast_arrays(np.asarray(mu, float),
                                              np.asarray(temperature, float))
        if np.any(temperature < 0):
            raise ValueError("temperature must be non-negative")
        e = self.energies
        e_rescaled = (e - self._b) / self._a
        prefactor = 2 * 4**2 / ((2 * self._a) ** 2)
        w = prefactor * _simpson_weights(e_rescaled) / \
            ((1 - e_rescaled ** 2) ** 2)
        factor = np.asarray(self._integral_factor)
        vals = factor.reshape(factor.shape[0], -1)
        out = _lib.fermi_sums(e, w, vals, mu.ravel(), temperature.ravel())
        return out.reshape(mu.shape + factor.shape[1:])

    def add_moments(self, num_moments=None, *, energy_resolution=None):
        """kwant/kpm.py:637-664 (recomputed on the device with the larger
        expansion; equal to a direct run with the final num_moments)."""
        if not ((num_moments is None) ^ (energy_resolution is None)):
            raise TypeError("either 'num_moments' or 'energy_resolution' "
                            "must be provided.")
        if energy_resolution:
            if energy_resolution <= 0:
                raise ValueError("'energy_resolution' must be positive")
            present_resolution = self._a * 1.6 / self.num_moments
            if present_resolution < energy_resolution:
                raise ValueError('Energy resolution is already smaller '
                                 'than the requested resolution')
            num_moments = math.ceil((1.6 * self._a) / energy_resolution)
        if (num_moments is None or num_moments <= 0
                or num_moments != int(num_moments)):
            raise ValueError("'num_moments' must be a positive integer")
        self.num_moments += int(num_moments)
        self._compute()

    def add_vectors(self, num_vectors=None):
        """kwant/kpm.py:666-683."""
        self._vector_factory.add_vectors(num_vectors)
        self._compute()


def _velocity(hamiltonian, params, op_type, positions):
    """kwant/kpm.py:1042-1085: v = H o i (x_col - x_row) for a direction,
    or the given operator / matrix."""
    directions = dict(x=0, y=1, z=2)
    if _is_local_operator(op_type):
        return op_type
    if isinstance(op_type, str):
        direction = directions[op_type]
        if _is_system(hamiltonian):
            operator, norbs, norbs = hamiltonian.hamiltonian_submatrix(
                params=params, sparse=True, return_norb=True)
            if hasattr(hamiltonian, 'orbital_positions'):
                positions = hamiltonian.orbital_positions()
            else:
                positions = np.vstack([[hamiltonian.pos(i)] * norb
                                       for i, norb in enumerate(norbs)])
        elif positions is not None:
            operator = coo_matrix(hamiltonian, copy=True)
        positions = np.asarray(positions, dtype=float)
        operator = coo_matrix(operator)
        displacements = positions[operator.col] - positions[operator.row]
        if direction > displacements.shape[1]:
            raise ValueError("{} is not an allowed direction.".format(op_type))
        operator.data = operator.data * (1j * displacements[:, direction])
        return operator.tocsr()
    try:
        return csr_matrix(op_type)
    except Exception:
        raise ValueError("Velocity operator must be provided as a matrix, "
                         "a kwant operator, or a direction.")


def conductivity(hamiltonian, alpha='x', beta='x', positions=None, **kwargs):
    """Kubo-Bastin conductivity tensor element (kwant/kpm.py:763-847)."""
    if positions is None and not _is_system(hamiltonian):
        raise ValueError("If 'hamiltonian' is a matrix, positions "
                         "must be provided")
    params = kwargs.get('params')
    alpha = _velocity(hamiltonian, params, alpha, positions)
    beta = _velocity(hamiltonian, params, beta, positions)
    return Correlator(hamiltonian, operator1=alpha, operator2=beta, **kwargs)
