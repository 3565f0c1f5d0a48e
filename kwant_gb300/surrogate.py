"""Learned moment surrogate for KPM parameter sweeps.

A parameter sweep of the DOS (e.g. disorder strength W, flux and a staggered
mass on one lattice) runs the full Chebyshev recursion once per point.  This
module puts a learned map in front of it:

``MomentSweep``
    the plain sweep: one device-resident Hamiltonian family
    (``HamiltonianFamily``; ``kpm_family_point`` regenerates H on the device
    per point) and one block of random-phase vectors, rewound per point; the
    moments of every point are those of ``kwant.kpm.SpectralDensity`` with
    fixed rescaling (a, b) for the whole parameter box and the same vectors
    at every point (kwant/kpm.py:163-252, :378-388).
``MomentSurrogate``
    an ensemble of small MLPs (parameters -> normalised moments mu_n / N),
    trained on the device by the library's own forward / backward / Adam
    kernels (``kpm_mlp_*``) on moments the plain sweep produced.  The spread
    of the members' DOS, times a factor calibrated on held-out KPM points,
    is its error estimate.
``SurrogateSweep``
    predictions where the estimated DOS error is at most ``tol`` and the
    plain KPM (the fallback and the error check) everywhere else.

DOS conventions: per site and per unit energy, Jackson kernel, at the
Chebyshev nodes x_k of 2M points with |x_k| <= ``x_max`` (energies
a x_k + b); errors are L-infinity over those energies.
"""

import itertools
import time

import numpy as np

from . import _lib
from .kpm import _rescale_ab, spectral_bounds

__all__ = ['MomentSweep', 'MomentSurrogate', 'SurrogateSweep',
           'dos_operator', 'random_points']


def random_points(box, n, seed):
    """n points drawn uniformly from the box ((lo, hi), ...) with
    RandomState(seed)."""
    rng = np.random.RandomState(seed)
    lo = np.array([b[0] for b in box], float)
    hi = np.array([b[1] for b in box], float)
    return lo + (hi - lo) * rng.random_sample((n, len(box)))


def dos_operator(num_moments, a, b, x_max=0.95):
    """Matrix A (K x M) and energies (K) with DOS(E_k) = A[k] . mu for
    normalised moments mu (mu_0 = 1): the Jackson-damped Chebyshev series
    (g_0 mu_0 + 2 sum_n g_n mu_n T_n(x_k)) / (pi a sqrt(1 - x_k^2)) at the
    Chebyshev nodes x_k = cos(pi (k + 1/2) / 2M) with |x_k| <= x_max (the
    reconstruction of kwant/kpm.py:1197-1222 written as a matrix)."""
    M = int(num_moments)
    g = _lib.kernel_weights(M, _lib.KERNEL_JACKSON)
    k = np.arange(2 * M)
    x = np.cos(np.pi * (k + 0.5) / (2 * M))[::-1]
    x = x[np.abs(x) <= x_max]
    n = np.arange(M)
    T = np.cos(np.outer(np.arccos(x), n))
    c = np.where(n == 0, 1.0, 2.0) * g
    A = T * c[None, :] / (np.pi * a * np.sqrt(1.0 - x * x))[:, None]
    return A, a * x + b


class MomentSweep:
    """Plain KPM over the points of a parameter family (see module doc).

    ``bounds``: (lmin, lmax) enclosing every point's spectrum; by default
    FP64 Lanczos bounds at the corners of the box (flux at its ends and
    middle), widened by ``margin`` of the width, then rescaled with
    ``eps`` like kwant/kpm.py:1174-1180.

    ``fresh_vectors``: False keeps one vector set for every point (the
    moments are then a deterministic function of the point); True draws an
    independent random-phase set per point on the device
    (``kpm_block_randomize``, keyed by ``rng`` and the running point count),
    so that the stochastic errors of different points are independent.
    """

    def __init__(self, family, box, num_moments=512, num_vectors=32,
                 precision='mixed', rng=1, bounds=None, eps=0.05,
                 margin=0.01, reorder=None, fresh_vectors=False):
        from .kpm import _precision
        self.family = family
        self.box = tuple(tuple(map(float, b)) for b in box)
        self.M = int(num_moments)
        self.R = int(num_vectors)
        if self.M % 2:
            raise ValueError('num_moments must be even')
        prec = _precision(precision)
        if bounds is None:
            bounds = self._corner_bounds(eps)
        lo, hi = bounds
        w = hi - lo
        self.bounds = (lo - margin * w, hi + margin * w)
        self.a, self.b = _rescale_ab(*self.bounds, eps)
        if reorder is None:
            reorder = prec == _lib.PREC_MIXED
        mid = [0.5 * (b0 + b1) for b0, b1 in self.box]
        self.handle = _lib.Handle(family.hamiltonian(*mid), self.a, self.b,
                                  prec, reorder=reorder)
        self.handle.family_set(family.base, family.theta, family.d1,
                               family.d2)
        N = family.shape[0]
        self.N = N
        rs = np.random.RandomState(rng)
        vecs = np.exp(2j * np.pi * rs.random_sample((self.R, N)))
        self.block = _lib.Block(self.handle, vecs, keep_a0=True)
        self.seconds = 0.0
        self.points_done = 0
        self.fresh = bool(fresh_vectors)
        self.seed = int(rng)

    def _corner_bounds(self, eps):
        (f0, f1), (w0, w1), (m0, m1) = self.box
        lo, hi = np.inf, -np.inf
        for pt in itertools.product((f0, 0.5 * (f0 + f1), f1), (w0, w1),
                                    (m0, m1)):
            l, h = spectral_bounds(self.family.hamiltonian(*pt), eps=eps)
            lo, hi = min(lo, l), max(hi, h)
        return lo, hi

    def moments(self, points, per_vector=False):
        """Normalised moments mu_n / N (mean over vectors, real part) of
        every point: P x M (or P x R x M complex if per_vector)."""
        points = np.atleast_2d(np.asarray(points, float))
        shape = (len(points), self.R, self.M) if per_vector else \
            (len(points), self.M)
        out = np.empty(shape, complex if per_vector else float)
        t0 = time.perf_counter()
        for i, p in enumerate(points):
            self.handle.family_point(*p)
            if self.fresh:
                self.block.randomize(self.seed * 1000003 +
                                     self.points_done + i)
            else:
                self.block.rewind()
            mom = self.block.dos_moments(0, self.M) / self.N
            out[i] = mom if per_vector else mom.mean(axis=0).real
        self.seconds += time.perf_counter() - t0
        self.points_done += len(points)
        return out

    def close(self):
        self.block.close()
        self.handle.close()


class MomentSurrogate:
    """Ensemble of MLPs mapping a parameter point to normalised moments.

    Inputs are mapped to [-1, 1] over ``box``, per coordinate either
    linearly or through a square root (``input_map`` entries 'linear' /
    'sqrt'; 'sqrt' suits a flux, whose Landau levels move like its square
    root).  Targets are the moments minus their training mean, weighted by
    each moment's weight in the DOS, c_n g_n (c_0 = 1, c_n = 2, g the
    Jackson kernel), and divided by one global scale: the training loss is
    then (up to a constant) the squared DOS error of the Chebyshev series,
    which measured 2x lower held-out DOS errors than standardising every
    moment (which amplifies the noise-dominated high moments).  Every member
    has the widths ``(len(box),) + hidden + (M,)`` and its own
    initialisation and shuffling seed.
    """

    def __init__(self, box, num_moments, hidden=(256, 256, 256), members=4,
                 seed=0, max_batch=4096, input_map=None):
        self.box = np.asarray(box, float)
        self.input_map = tuple(input_map or ('linear',) * len(self.box))
        if len(self.input_map) != len(self.box) or not set(
                self.input_map) <= {'linear', 'sqrt'}:
            raise ValueError("input_map: one 'linear' or 'sqrt' per input")
        self.M = int(num_moments)
        self.widths = (self.box.shape[0],) + tuple(hidden) + (self.M,)
        self.nets = [_lib.Mlp(self.widths, max_batch=max_batch,
                              seed=seed * 1000 + e) for e in range(members)]
        self.seed = seed
        self.scale = 1.0
        self.train_seconds = 0.0

    def _x(self, points):
        lo, hi = self.box[:, 0], self.box[:, 1]
        u = (np.asarray(points, float) - lo) / (hi - lo)
        for i, m in enumerate(self.input_map):
            if m == 'sqrt':
                u[:, i] = np.sqrt(np.clip(u[:, i], 0.0, None))
        return (2 * u - 1).astype(np.float32)

    def fit(self, points, moments, epochs=2000, batch=256, lr=1e-3,
            decay_stages=4):
        """Train every member with Adam: ``epochs`` split into
        ``decay_stages`` stages with the learning rate divided by 3 from one
        stage to the next.  Returns the members' last-epoch losses."""
        moments = np.asarray(moments, float)
        self.mean = moments.mean(axis=0)
        g = _lib.kernel_weights(self.M, _lib.KERNEL_JACKSON)
        w = np.where(np.arange(self.M) == 0, 1.0, 2.0) * np.abs(g)
        spread = np.abs(moments - self.mean).max()
        spread = spread / 3.0 if spread > 0 else 1.0
        self.std = spread / np.maximum(w, 1e-3)
        x = self._x(points)
        y = ((moments - self.mean) / self.std).astype(np.float32)
        t0 = time.perf_counter()
        losses = []
        per = max(1, epochs // decay_stages)
        for e, net in enumerate(self.nets):
            rate = lr
            for s in range(decay_stages):
                loss = net.train(x, y, batch, per, rate,
                                 seed=self.seed * 7919 + e * 31 + s)
                rate /= 3.0
            losses.append(loss)
        self.train_seconds += time.perf_counter() - t0
        return losses

    def predict_members(self, points):
        """Moments predicted by every member: E x P x M."""
        x = self._x(np.atleast_2d(points))
        return np.stack([net.forward(x).astype(np.float64) * self.std +
                         self.mean for net in self.nets])

    def predict(self, points, dos_op):
        """Ensemble-mean moments (P x M) and the estimated DOS error (P):
        ``scale`` times the largest (over energies) standard deviation of the
        members' DOS."""
        mem = self.predict_members(points)
        if len(self.nets) < 2:                        # no spread: no estimate
            return mem[0], np.full(mem.shape[1], np.inf)
        # the members' DOS and its spread on the device
        spread, _ = _lib.ensemble_dos(mem, np.ascontiguousarray(dos_op.T))
        return mem.mean(axis=0), self.scale * spread

    def calibrate(self, points, moments, dos_op, quantile=0.95):
        """Set ``scale`` so that the estimate covers the actual DOS error
        (against the given KPM moments) on ``quantile`` of the points."""
        mem = self.predict_members(points)
        spread, err = _lib.ensemble_dos(mem, np.ascontiguousarray(dos_op.T),
                                        ref=moments)
        if len(self.nets) < 2:
            self.scale = np.inf
            return err, np.full(err.shape, np.inf)
        self.scale = float(np.quantile(err / np.maximum(spread, 1e-300),
                                       quantile))
        return err, spread

    def close(self):
        for n in self.nets:
            n.close()


class SurrogateSweep:
    """Surrogate first, KPM where the surrogate's estimated DOS error is
    above ``tol``."""

    def __init__(self, surrogate, kpm_sweep, dos_op, tol=1e-4):
        self.surrogate = surrogate
        self.kpm = kpm_sweep
        self.dos_op = dos_op
        self.tol = float(tol)

    def run(self, points):
        """Moments of every point (P x M), the mask of points answered by
        the surrogate, and timings (seconds) of both parts."""
        points = np.atleast_2d(np.asarray(points, float))
        t0 = time.perf_counter()
        mom, est = self.surrogate.predict(points, self.dos_op)
        t1 = time.perf_counter()
        accept = est <= self.tol
        if not accept.all():
            mom[~accept] = self.kpm.moments(points[~accept])
        t2 = time.perf_counter()
        return mom, accept, {'surrogate_s': t1 - t0, 'kpm_s': t2 - t1,
                             'estimate': est}
