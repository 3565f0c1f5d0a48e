"""Batched KPM: many systems (disorder realisations, parameter points,
lattices of uneven size) in one set of launches per Chebyshev step, captured
in a CUDA graph (``kpm_batch_*`` in include/kwant_gb300.h).

This replaces looping ``kwant.kpm.SpectralDensity`` (kwant/kpm.py:163-252)
over realisations.  Matrices are block-sparse with 4 x 4 blocks (4-orbital
models such as the Wilson-Dirac topological insulator).  The random-phase
vectors are drawn on the device from a counter-based generator whose stream
``random_phase_vectors`` reproduces on the host.

Two precisions:

* ``'single'``: plain complex64 vectors with FP64 moment accumulation; every
  system advances in one launch per step, and the whole run is one CUDA
  graph.  On the 32-system Wilson-Dirac workload (M = 1024) the per-orbital
  DOS is 5e-5 off the FP64 path at the outermost Chebyshev node.
* ``'mixed'``: the compensated single-system step (complex64 plus bfloat16
  corrections, error-free FP32 sums; the DOS gate of 1e-5), one resident
  handle and block per system, advanced system after system, with the same
  starting vectors as ``'single'``.
"""

import time

import numpy as np
import scipy.sparse as sp

from . import _lib

__all__ = ['BatchedDOS', 'random_phase_vectors', 'wilson_dirac_disorder',
           'mix64']

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def mix64(z):
    """SplitMix64 finalizer (Steele, Lea & Flood 2014), vectorised over a
    uint64 array; the same function the device generator uses."""
    with np.errstate(over='ignore'):
        z = np.asarray(z, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def random_phase_vectors(seed, system, num_vectors, num_orbitals):
    """The starting vectors the device uses for system number ``system`` of
    a batch created with ``seed``: (R, N) complex64, entries exp(2 pi i u),
    u = top 24 bits of SplitMix64(SplitMix64(key ^ r) + n) / 2^24, key =
    SplitMix64(seed ^ (system << 32))."""
    key = mix64(np.uint64(seed) ^ (np.uint64(system) << np.uint64(32)))
    out = np.empty((num_vectors, num_orbitals), dtype=np.complex64)
    n = np.arange(num_orbitals, dtype=np.uint64)
    for r in range(num_vectors):
        with np.errstate(over='ignore'):
            h = mix64(mix64(key ^ np.uint64(r)) + n)
        u = (h >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)
        ang = 2.0 * np.pi * u.astype(np.float64)
        out[r] = (np.cos(ang) + 1j * np.sin(ang)).astype(np.complex64)
    return out


def wilson_dirac_disorder(seed, L, W):
    """Onsite disorder w of every site of a device-generated Wilson-Dirac
    system: w = W (u - 1/2), u = SplitMix64(SplitMix64(SplitMix64(seed)
    ^ 0xD15C0) + site) / 2^64 (53 bits)."""
    key = mix64(mix64(np.uint64(seed)) ^ np.uint64(0xD15C0))
    s = np.arange(L ** 3, dtype=np.uint64)
    with np.errstate(over='ignore'):
        h = mix64(key + s)
    u = (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return W * (u - 0.5)


def _rescale(lmin, lmax, eps):
    tol = eps / 2
    a = np.abs(lmax - lmin) / (2. - eps)
    b = (lmax + lmin) / 2.
    if lmax - lmin <= abs(lmax + lmin) * tol / 2:
        raise ValueError('The Hamiltonian has a single eigenvalue')
    return a, b


class BatchedDOS:
    """DOS of many 4-orbital systems at once.

    Parameters
    ----------
    num_vectors, num_moments : int (num_moments even)
    seed : int, seed of the device vector generator
    eps : float, spectral margin as in kwant.kpm (kwant/kpm.py:1174)
    precision : 'single' (default) or 'mixed' (see the module docstring)
    """

    def __init__(self, num_vectors=256, num_moments=1024, seed=0, eps=0.05,
                 precision='single'):
        if precision not in ('single', 'mixed'):
            raise ValueError("precision must be 'single' or 'mixed'")
        if int(num_moments) <= 0 or int(num_moments) % 2:
            raise ValueError('num_moments must be a positive even integer')
        self.num_vectors = int(num_vectors)
        self.num_moments = int(num_moments)
        self.eps = eps
        self.precision = precision
        self.seed = int(seed)
        self.scales = []
        if precision == 'single':
            self._b = _lib.Batch(num_vectors, num_moments, seed)
        else:
            self._mats = []        # host CSR per system
            self._sys = []         # (handle, block) per system, on first run
            self._last = (0.0, 0)

    def add_matrix(self, ham, bounds):
        """A system given as a (4-orbital) sparse matrix and its spectral
        bounds (lmin, lmax)."""
        a, b = _rescale(bounds[0], bounds[1], self.eps)
        if self.precision == 'single':
            self._b.add_bsr(ham, a, b)
        else:
            self._add_host(sp.csr_matrix(ham))
        self.scales.append((a, b))

    def add_wilson_dirac(self, L, m=1.5, W=0.0, seed=0, bounds=None):
        """An L^3 Wilson-Dirac system, generated on the device ('single')
        or assembled on the host with the device generator's disorder
        ('mixed').  Default bounds: the Gershgorin bound
        |E| <= |m - 3| + W/2 + 6."""
        if bounds is None:
            g = abs(m - 3) + W / 2 + 6.0
            bounds = (-g, g)
        a, b = _rescale(bounds[0], bounds[1], self.eps)
        if self.precision == 'single':
            self._b.add_wilson_dirac(L, m, W, seed, a, b)
        else:
            self._add_host(wilson_dirac_matrix(L, m, W, seed))
        self.scales.append((a, b))

    def _add_host(self, ham):
        if self._sys:
            raise RuntimeError('BatchedDOS: batch already run')
        if ham.shape[0] % 4:
            raise ValueError('the batch holds 4-orbital systems')
        self._mats.append(ham.tocsr())

    def moments(self):
        """(systems, M) complex128 moments, mean over the vectors."""
        if self.precision == 'single':
            return self._b.run()
        t0 = time.perf_counter()
        launches0 = _lib.launch_count()
        if not self._sys:
            made = []
            try:
                for s, H in enumerate(self._mats):
                    a, b = self.scales[s]
                    h = _lib.Handle(H, a, b, _lib.PREC_MIXED)
                    made.append((h, None))
                    made[-1] = (h, _lib.Block(h, None,
                                              num_vectors=self.num_vectors))
            except BaseException:
                for h, blk in made:      # nothing half-built stays resident
                    if blk is not None:
                        blk.close()
                    h.close()
                raise
            self._sys = made
        out = np.empty((len(self._sys), self.num_moments), complex)
        for s, (h, blk) in enumerate(self._sys):
            # the device generator of 'single' with this system's key: the
            # block keys its stream by mix64(seed ^ 0x5EEDB10C), the batch
            # by mix64(seed ^ (system << 32)); storage order = orbital order
            blk.randomize(self.seed ^ (s << 32) ^ 0x5EEDB10C)
            out[s] = blk.dos_moments(0, self.num_moments).mean(axis=0)
        self._last = ((time.perf_counter() - t0) * 1e3,
                      _lib.launch_count() - launches0)
        return out

    def densities(self, moments=None):
        """Densities at the 2M Chebyshev nodes of every system (Jackson
        kernel, device reconstruction) and the energies."""
        mom = self.moments() if moments is None else moments
        from .kpm import _chebyshev_nodes
        nodes = _chebyshev_nodes(2 * self.num_moments)
        rho, en = [], []
        for s, (a, b) in enumerate(self.scales):
            m = mom[s][None, :, None]
            is_real = bool(np.all(np.abs(m.imag) < 100 * 2.220446049250313e-16))
            _, r = _lib.reconstruct(m, True, is_real, a, _lib.KERNEL_JACKSON,
                                    4.0, nodes)
            rho.append(r[:, 0].real if is_real else r[:, 0])
            en.append(a * nodes + b)
        return np.array(en), np.array(rho)

    def stats(self):
        """'single': (device ms of the last run, graph kernel nodes,
        vectors per lane chosen by the autotuner); 'mixed': (wall ms of the
        last run, kernel launches of that run, 2)."""
        if self.precision == 'mixed':
            return self._last[0], self._last[1], 2
        return self._b.stats()

    def step_format(self):
        """Step kernel chosen by the autotuner at the first run:
        ``(format, ell_width)`` with format 0 = dense 4 x 4 blocks, 1 =
        orbital-row ELL of width ell_width, 2 = sparse blocks staged in
        shared memory; 'mixed': ``(3, 0)``, the compensated ELL step."""
        if self.precision == 'mixed':
            return 3, 0
        return self._b.step_format()

    def work_order(self):
        """'single': the autotuner's work order ('partition' or 'group',
        see kpm_batch_order); 'mixed': None (systems run one by one)."""
        if self.precision == 'mixed':
            return None
        return self._b.work_order()

    def close(self):
        """Free the device state of a 'mixed' batch."""
        if self.precision == 'mixed':
            for h, blk in self._sys:
                blk.close()
                h.close()
            self._sys = []


def wilson_dirac_matrix(L, m=1.5, W=0.0, seed=0):
    """Host CSR of the L^3 Wilson-Dirac system that
    ``add_wilson_dirac(L, m, W, seed)`` generates on the device (the
    lattices builder's hoppings and onsite mass, the device generator's
    disorder)."""
    from . import lattices
    H = lattices.wilson_dirac_cubic(L, m=m, W=0.0).hamiltonian_submatrix(
        sparse=True).tocsr()
    w = wilson_dirac_disorder(seed, L, W)
    return (H + sp.diags(np.repeat(w, 4))).tocsr()
