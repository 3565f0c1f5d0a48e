"""ctypes binding of ``libkwant_gb300.so`` (the C ABI in include/kwant_gb300.h).

There is no CPU fallback: importing this module without the built library
raises ``ImportError``, and every compute call without a CUDA device raises
``KPMCudaError``.
"""

import ctypes as C
import weakref
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# KWANT_GB300_LIB may name another build of the library (the bounds-checked
# variant of kwant_gb300.build)
LIB_PATH = os.environ.get('KWANT_GB300_LIB') or \
    os.path.join(_HERE, 'libkwant_gb300.so')

KPM_OK = 0
KPM_EINVAL = -1
KPM_ECUDA = -2
KPM_ENOMEM = -3
KPM_EDIVERGED = -4
KPM_ETIMEOUT = -5
KPM_ESTATE = -6
KPM_EUNSUPPORTED = -7

PREC_FP64 = 0
PREC_MIXED = 1
# host-side code: KPM_PREC_MIXED with KPM_FLAG_PLAIN_C64 (plain complex64
# DOS recursion, no compensation)
PREC_SINGLE = 2
KERNEL_NONE = 0
KERNEL_JACKSON = 1
KERNEL_LORENTZ = 2
FLAG_REORDER = 1
FLAG_PLAIN_C64 = 2
DEBUG_WAIT_NS = 1
DEBUG_STALL_TMA = 2


class KPMError(RuntimeError):
    pass


class KPMCudaError(KPMError):
    pass


class KPMStateError(KPMError):
    pass


class KPMUnsupported(KPMError, NotImplementedError):
    pass


class KPMDiverged(KPMError):
    pass


class CsrDesc(C.Structure):
    _fields_ = [('rows', C.c_int64), ('nnz', C.c_int64),
                ('indptr', C.c_void_p), ('indices', C.c_void_p),
                ('data', C.c_void_p)]


class BsrDesc(C.Structure):
    _fields_ = [('block_rows', C.c_int64), ('nnzb', C.c_int64),
                ('indptr', C.c_void_p), ('indices', C.c_void_p),
                ('data', C.c_void_p)]


class OpDesc(C.Structure):
    _fields_ = [('num_terms', C.c_int64), ('num_outputs', C.c_int64),
                ('num_chunks', C.c_int64), ('term_row', C.c_void_p),
                ('bra_ptr', C.c_void_p), ('bra_col', C.c_void_p),
                ('bra_val', C.c_void_p), ('chunk_ptr', C.c_void_p),
                ('chunk_out', C.c_void_p), ('real0', C.c_int32)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            'kwant_gb300 CUDA library not built (%s missing); run '
            '"python -m kwant_gb300.build" (needs nvcc, sm_103a)' % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    I64 = C.c_int64
    D = C.c_double
    I = C.c_int
    sigs = {
        'kpm_version': [],
        'kpm_last_error': [C.c_char_p, C.c_size_t],
        'kpm_device_count': [P],
        'kpm_create': [P, D, D, I, P],
        'kpm_create_ex': [P, D, D, I, I, P],
        'kpm_set_stream': [P, P],
        'kpm_get_stream': [P, P],
        'kpm_synchronize': [P],
        'kpm_destroy': [P],
        'kpm_block_create': [P, P, I64, I, P],
        'kpm_block_rewind': [P],
        'kpm_block_randomize': [P, C.c_uint64],
        'kpm_block_destroy': [P],
        'kpm_block_state': [P, P, P],
        'kpm_block_checkpoint': [P, P, P, P],
        'kpm_block_restore': [P, I64, I, P, P, P],
        'kpm_block_dos_moments': [P, I64, I64, P],
        'kpm_op_create': [P, P, P],
        'kpm_op_destroy': [P],
        'kpm_block_op_moments': [P, P, I64, I64, P],
        'kpm_op_apply': [P, P, P, P],
        'kpm_dos': [P, D, D, I, P, I64, I64, I, P, P, P],
        'kpm_reconstruct': [I64, I64, I64, P, I, I, D, I, D, P, P, P],
        'kpm_kernel_weights': [I64, I, D, P],
        'kpm_chebval': [I64, I64, P, I64, P, P],
        'kpm_bounds': [P, P, D, I, P, P, P],
        'kpm_handle_matvec': [P, P, P],
        'kpm_correlator_moments': [P, D, D, P, P, P, I64, I64, I, I, P],
        'kpm_integral_factor': [I64, P, P, P, P],
        'kpm_fermi_sums': [I64, P, P, I64, P, I64, P, P, P],
        'kpm_ensemble_dos': [I64, I64, I64, I64, P, P, P, P, P],
        'kpm_last_kernel_ms': [P, P],
        'kpm_dos_moments_noalloc': [P, D, D, I, P, I64, I64, P, P, P],
        'kpm_last_gemm': [P, P, P],
        'kpm_batch_create': [I64, I64, C.c_uint64, P],
        'kpm_batch_add_bsr': [P, P, D, D],
        'kpm_batch_add_wilson_dirac': [P, I64, D, D, C.c_uint64, D, D],
        'kpm_batch_run': [P, P],
        'kpm_batch_stats': [P, P, P, P],
        'kpm_batch_format': [P, P, P],
        'kpm_batch_order': [P, P],
        'kpm_batch_destroy': [P],
        'kpm_profile': [P, I],
        'kpm_profile_read': [P, P, P],
        'kpm_launch_count': [P],
        'kpm_debug_set': [I, I64],
        'kpm_build_checks': [P],
        'kpm_family_set': [P, P, P, P, P],
        'kpm_family_point': [P, D, D, D],
        'kpm_mlp_create': [I, P, I, C.c_uint64, P],
        'kpm_mlp_num_params': [P, P],
        'kpm_mlp_get_params': [P, P],
        'kpm_mlp_set_params': [P, P],
        'kpm_mlp_forward': [P, P, I64, P],
        'kpm_mlp_gradients': [P, P, P, I64, P, P],
        'kpm_mlp_train': [P, P, P, I64, I, I64, D, C.c_uint64, P],
        'kpm_mlp_destroy': [P],
    }
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    return lib


lib = _load()


def last_error():
    buf = C.create_string_buffer(1024)
    lib.kpm_last_error(buf, len(buf))
    return buf.value.decode(errors='replace')


def check(status):
    if status == KPM_OK:
        return
    msg = last_error()
    if status == KPM_EINVAL:
        raise ValueError(msg)
    if status == KPM_ECUDA or status == KPM_ENOMEM:
        raise KPMCudaError(msg)
    if status == KPM_ESTATE:
        raise KPMStateError(msg)
    if status == KPM_EUNSUPPORTED:
        raise KPMUnsupported(msg)
    if status == KPM_EDIVERGED:
        raise KPMDiverged(msg)
    raise KPMError('status %d: %s' % (status, msg))


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def debug_set(key, value):
    """kpm_debug_set: process-wide diagnostics (DEBUG_WAIT_NS: bound of
    the tensor-core kernels' mbarrier waits; DEBUG_STALL_TMA: tests only,
    their TMA producers issue no loads)."""
    check(lib.kpm_debug_set(int(key), int(value)))


def build_checks():
    """True when the loaded library is the bounds-checked build."""
    on = C.c_int(0)
    check(lib.kpm_build_checks(C.byref(on)))
    return bool(on.value)


def device_count():
    n = C.c_int(0)
    check(lib.kpm_device_count(C.byref(n)))
    return n.value


def launch_count():
    n = C.c_int64(0)
    check(lib.kpm_launch_count(C.byref(n)))
    return n.value


class Csr:
    """Host CSR arrays kept alive together with their C descriptor."""

    def __init__(self, mat):
        import scipy.sparse as sp
        m = sp.csr_matrix(mat)
        if m.shape[0] != m.shape[1]:
            raise ValueError('matrix must be square')
        self.shape = m.shape
        self.indptr = np.ascontiguousarray(m.indptr, dtype=np.int32)
        self.indices = np.ascontiguousarray(m.indices, dtype=np.int32)
        self.data = np.ascontiguousarray(m.data, dtype=np.complex128)
        self.nnz = int(self.data.shape[0])
        self.desc = CsrDesc(m.shape[0], self.nnz, ptr(self.indptr),
                            ptr(self.indices), ptr(self.data))

    def ref(self):
        return C.byref(self.desc)


def c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


class Handle:
    """A Hamiltonian resident on the device with its rescaling (a, b)."""

    def __init__(self, csr, a, b, precision, reorder=False):
        if not isinstance(csr, Csr):
            csr = Csr(csr)
        self.csr = csr
        self.a, self.b, self.precision = float(a), float(b), precision
        self.N = csr.shape[0]
        self.reorder = bool(reorder)
        h = C.c_void_p()
        self._children = weakref.WeakSet()
        flags = FLAG_REORDER if reorder else 0
        cprec = precision
        if precision == PREC_SINGLE:
            cprec, flags = PREC_MIXED, flags | FLAG_PLAIN_C64
        check(lib.kpm_create_ex(csr.ref(), self.a, self.b, cprec, flags,
                                C.byref(h)))
        self._h = h

    @property
    def ptr(self):
        return self._h

    def stream(self):
        s = C.c_void_p()
        check(lib.kpm_get_stream(self._h, C.byref(s)))
        return s.value

    def last_kernel_ms(self):
        ms = C.c_double()
        check(lib.kpm_last_kernel_ms(self._h, C.byref(ms)))
        return ms.value

    def last_gemm(self):
        ms, fl = C.c_double(), C.c_double()
        check(lib.kpm_last_gemm(self._h, C.byref(ms), C.byref(fl)))
        return ms.value, fl.value

    def profile(self, enable=True):
        check(lib.kpm_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        n, ms = C.c_int64(), C.c_double()
        check(lib.kpm_profile_read(self._h, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def matvec(self, x):
        x = c128(x)
        y = np.empty_like(x)
        check(lib.kpm_handle_matvec(self._h, ptr(x), ptr(y)))
        return y

    def family_set(self, base, theta, d1, d2):
        """Coefficient matrices of H(phi, s1, s2) = base .* exp(i phi
        theta) + s1 d1 + s2 d2 (scipy CSR, the handle's structure)."""
        self._family = [m if isinstance(m, Csr) else Csr(m)
                        for m in (base, theta, d1, d2)]
        check(lib.kpm_family_set(self._h, *[m.ref() for m in self._family]))

    def family_point(self, phi, s1, s2):
        check(lib.kpm_family_point(self._h, float(phi), float(s1),
                                   float(s2)))

    def close(self):
        # blocks and operators hold device state tied to the handle: free
        # them first (they are weakly tracked; see Block.close for the
        # order-free case of garbage collection at interpreter exit)
        for child in list(getattr(self, '_children', ())):
            child.close()
        if getattr(self, '_h', None):
            lib.kpm_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Block:
    """R vectors and their recursion state on the device."""

    def __init__(self, handle, vecs, keep_a0=True, num_vectors=None):
        """vecs: (R, N) starting vectors, or None with num_vectors = R
        for a block of zero vectors on the device (then `randomize`)."""
        self.handle = handle
        if vecs is None:
            if num_vectors is None or int(num_vectors) <= 0:
                raise ValueError('num_vectors must be positive')
            self.R = int(num_vectors)
            vp = None
        else:
            vecs = c128(np.atleast_2d(vecs))
            self.R = vecs.shape[0]
            if vecs.shape[1] != handle.N:
                raise ValueError('vector length does not match the '
                                 'Hamiltonian')
            vp = ptr(vecs)
        b = C.c_void_p()
        check(lib.kpm_block_create(handle.ptr, vp, self.R,
                                   1 if keep_a0 else 0, C.byref(b)))
        self._b = b
        handle._children.add(self)

    def dos_moments(self, m_start, m_end, diverged='raise'):
        """R x (m_end - m_start) DOS moments.  A recursion that diverged
        (KPM_EDIVERGED: spectral bounds that leave eigenvalues outside)
        raises KPMDiverged, or with diverged='return' returns the moments
        and keeps the message in self.diverged."""
        out = np.empty((self.R, m_end - m_start), dtype=np.complex128)
        st = lib.kpm_block_dos_moments(self._b, m_start, m_end, ptr(out))
        self.diverged = None
        if st == KPM_EDIVERGED and diverged == 'return':
            self.diverged = last_error()
            return out
        check(st)
        return out

    def op_moments(self, op, m_start, m_end):
        out = np.empty((self.R, m_end - m_start, op.W), dtype=np.complex128)
        check(lib.kpm_block_op_moments(self._b, op.ptr, m_start, m_end,
                                       ptr(out)))
        return out

    def rewind(self):
        check(lib.kpm_block_rewind(self._b))

    def randomize(self, seed):
        """New random-phase starting vectors generated on the device."""
        check(lib.kpm_block_randomize(self._b,
                                      C.c_uint64(int(seed) & (2**64 - 1))))

    def state(self):
        prev = np.empty((self.R, self.handle.N), dtype=np.complex128)
        cur = np.empty_like(prev)
        check(lib.kpm_block_state(self._b, ptr(prev), ptr(cur)))
        return prev, cur

    def checkpoint(self):
        """(steps_done, mode, mu01 (R x 2), alpha_prev, alpha_cur); the
        vectors are None before the first step."""
        steps, mode = C.c_int64(), C.c_int()
        mu01 = np.empty((self.R, 2), dtype=np.complex128)
        check(lib.kpm_block_checkpoint(self._b, C.byref(steps),
                                       C.byref(mode), ptr(mu01)))
        prev = cur = None
        if steps.value > 0:
            prev, cur = self.state()
        return steps.value, mode.value, mu01, prev, cur

    def restore(self, steps, mode, mu01, prev=None, cur=None):
        mu01 = c128(mu01)
        if steps > 0:
            prev, cur = c128(prev), c128(cur)
            check(lib.kpm_block_restore(self._b, int(steps), int(mode),
                                        ptr(prev), ptr(cur), ptr(mu01)))
        else:
            check(lib.kpm_block_restore(self._b, 0, int(mode), None, None,
                                        ptr(mu01)))

    def close(self):
        if getattr(self, '_b', None):
            # a block outliving its handle (finalizers of a reference cycle
            # run in any order) must not touch the destroyed handle
            if getattr(self.handle, '_h', None):
                lib.kpm_block_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()


class Op:
    """A lowered sesquilinear operator on the device."""

    def __init__(self, handle, lowered):
        self.handle = handle
        self.low = lowered
        self.W = int(lowered.num_outputs)
        d = OpDesc(lowered.num_terms, lowered.num_outputs,
                   lowered.num_chunks, ptr(lowered.term_row),
                   ptr(lowered.bra_ptr), ptr(lowered.bra_col),
                   ptr(lowered.bra_val), ptr(lowered.chunk_ptr),
                   ptr(lowered.chunk_out), int(lowered.real0))
        o = C.c_void_p()
        check(lib.kpm_op_create(handle.ptr, C.byref(d), C.byref(o)))
        self._o = o
        handle._children.add(self)

    @property
    def ptr(self):
        return self._o

    def apply(self, bra, ket):
        bra, ket = c128(bra), c128(ket)
        out = np.empty(self.W, dtype=np.complex128)
        check(lib.kpm_op_apply(self._o, ptr(bra), ptr(ket), ptr(out)))
        return out

    def close(self):
        if getattr(self, '_o', None):
            if getattr(self.handle, '_h', None):
                lib.kpm_op_destroy(self._o)
            self._o = None

    def __del__(self):
        self.close()


def reconstruct(moments, mean, is_real, a, kernel, lorentz_l, nodes):
    """moments: (R, M, W) complex128 -> (gammas, densities), each
    (2M, W') complex128."""
    moments = c128(moments)
    R, M, W = moments.shape
    Wo = W if mean else R * W
    gam = np.empty((2 * M, Wo), dtype=np.complex128)
    rho = np.empty_like(gam)
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    check(lib.kpm_reconstruct(R, M, W, ptr(moments), 1 if mean else 0,
                              1 if is_real else 0, float(a), kernel,
                              float(lorentz_l), ptr(nodes), ptr(gam),
                              ptr(rho)))
    return gam, rho


def chebval(x, coefs):
    """numpy.polynomial.chebyshev.chebval(x, coefs) (tensor form) on the
    device: coefs (M, ...) complex, x any shape -> coefs.shape[1:] +
    x.shape complex."""
    c = np.asarray(coefs, dtype=np.complex128)
    M = c.shape[0]
    tail = c.shape[1:]
    W = int(np.prod(tail)) if tail else 1
    c2 = np.ascontiguousarray(c.reshape(M, W))
    xs = np.asarray(x, dtype=np.float64)
    xf = np.ascontiguousarray(xs.reshape(-1))
    out = np.empty((xf.size, W), dtype=np.complex128)
    check(lib.kpm_chebval(M, W, ptr(c2), xf.size, ptr(xf), ptr(out)))
    return out.T.reshape(tail + xs.shape)


def kernel_weights(M, kernel, lorentz_l=4.0):
    g = np.empty(M, dtype=np.float64)
    check(lib.kpm_kernel_weights(M, kernel, float(lorentz_l), ptr(g)))
    return g


def bounds(csr, v0, tol, max_iter=1000):
    if not isinstance(csr, Csr):
        csr = Csr(csr)
    v0 = c128(v0)
    lo, hi, it = C.c_double(), C.c_double(), C.c_int()
    check(lib.kpm_bounds(csr.ref(), ptr(v0), float(tol), int(max_iter),
                         C.byref(lo), C.byref(hi), C.byref(it)))
    return lo.value, hi.value, it.value


def correlator_moments(handle, a2, b2, v_alpha, v_beta, vecs, M, gemm=2,
                       per_vector=False):
    va = v_alpha if isinstance(v_alpha, Csr) else Csr(v_alpha)
    vb = v_beta if isinstance(v_beta, Csr) else Csr(v_beta)
    vecs = c128(np.atleast_2d(vecs))
    R = vecs.shape[0]
    shape = (R, M, M) if per_vector else (M, M)
    out = np.empty(shape, dtype=np.complex128)
    check(lib.kpm_correlator_moments(handle.ptr, float(a2), float(b2),
                                     va.ref(), vb.ref(), ptr(vecs), R, M,
                                     int(gemm), 1 if per_vector else 0,
                                     ptr(out)))
    return out


def fermi_sums(energies, weights, values, mu=None, temperature=None):
    """sum_k weights[k] * f(energies[k]; mu, T) * values[k, :] on the
    device for every (mu, T) point (f = 1 without mu): values (n, W)
    complex, mu / temperature 1-D of length P -> (P, W) complex128."""
    e = np.ascontiguousarray(energies, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    v = c128(values)
    n, W = v.shape
    if mu is None:
        P, pm, pt = 1, None, None
    else:
        pm = np.ascontiguousarray(mu, dtype=np.float64).ravel()
        pt = np.ascontiguousarray(temperature, dtype=np.float64).ravel()
        if pm.shape != pt.shape:
            raise ValueError('mu and temperature must have the same size')
        if np.any(pt < 0):
            raise ValueError('temperature must be non-negative')
        P = pm.size
    out = np.empty((P, W), dtype=np.complex128)
    check(lib.kpm_fermi_sums(n, ptr(e), ptr(w), W, ptr(v), P,
                             ptr(pm) if pm is not None else None,
                             ptr(pt) if pt is not None else None, ptr(out)))
    return out


def integral_factor(mu, g, nodes):
    mu = c128(mu)
    M = mu.shape[0]
    g = np.ascontiguousarray(g, dtype=np.float64)
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    out = np.empty(2 * M, dtype=np.complex128)
    check(lib.kpm_integral_factor(M, ptr(mu), ptr(g), ptr(nodes), ptr(out)))
    return out


def dos(csr, a, b, precision, vecs, M, kernel=KERNEL_JACKSON):
    if not isinstance(csr, Csr):
        csr = Csr(csr)
    vecs = c128(np.atleast_2d(vecs))
    R = vecs.shape[0]
    mom = np.empty((R, M), dtype=np.complex128)
    gam = np.empty(2 * M, dtype=np.complex128)
    rho = np.empty(2 * M, dtype=np.complex128)
    check(lib.kpm_dos(csr.ref(), float(a), float(b), precision, ptr(vecs), R,
                      M, kernel, ptr(mom), ptr(gam), ptr(rho)))
    return mom, gam, rho


def ensemble_dos(members, At, ref=None):
    """Surrogate ensemble DOS on the device (kpm_ensemble_dos): members
    (E, P, M) moments, At (M, K) projection to K energies.  Returns the
    spread (P) and, with ref (P, M), the error of the member mean (P)."""
    mem = np.ascontiguousarray(members, dtype=np.float64)
    At = np.ascontiguousarray(At, dtype=np.float64)
    E, P, M = mem.shape
    if not 0 < E <= 8:
        raise ValueError('the device ensemble takes 1 to 8 members')
    if At.shape[0] != M:
        raise ValueError('At must be (num_moments, energies)')
    K = At.shape[1]
    spread = np.empty(P)
    err = None
    rp = None
    if ref is not None:
        rp = np.ascontiguousarray(ref, dtype=np.float64)
        if rp.shape != (P, M):
            raise ValueError('ref must be (points, num_moments)')
        err = np.empty(P)
    check(lib.kpm_ensemble_dos(E, P, M, K, ptr(mem), ptr(At), ptr(rp),
                               ptr(spread), ptr(err)))
    return spread, err


class Batch:
    """Many systems advanced together (kpm_batch_* C ABI)."""

    def __init__(self, num_vectors, num_moments, seed=0):
        b = C.c_void_p()
        check(lib.kpm_batch_create(int(num_vectors), int(num_moments),
                                   C.c_uint64(int(seed) & (2**64 - 1)),
                                   C.byref(b)))
        self._b = b
        self.R, self.M = int(num_vectors), int(num_moments)
        self.num_systems = 0
        self._keep = []

    def add_bsr(self, bsr, a, b):
        import scipy.sparse as sp
        m = sp.bsr_matrix(bsr, blocksize=(4, 4))
        m.sort_indices()
        indptr = np.ascontiguousarray(m.indptr, dtype=np.int32)
        indices = np.ascontiguousarray(m.indices, dtype=np.int32)
        data = np.ascontiguousarray(m.data, dtype=np.complex128)
        d = BsrDesc(m.shape[0] // 4, len(indices), ptr(indptr), ptr(indices),
                    ptr(data))
        check(lib.kpm_batch_add_bsr(self._b, C.byref(d), float(a), float(b)))
        self.num_systems += 1

    def add_wilson_dirac(self, L, m, W, seed, a, b):
        check(lib.kpm_batch_add_wilson_dirac(
            self._b, int(L), float(m), float(W),
            C.c_uint64(int(seed) & (2**64 - 1)), float(a), float(b)))
        self.num_systems += 1

    def run(self):
        out = np.empty((self.num_systems, self.M), dtype=np.complex128)
        check(lib.kpm_batch_run(self._b, ptr(out)))
        return out

    def stats(self):
        ms, nodes, vpl = C.c_double(), C.c_int64(), C.c_int()
        check(lib.kpm_batch_stats(self._b, C.byref(ms), C.byref(nodes),
                                  C.byref(vpl)))
        return ms.value, nodes.value, vpl.value

    def step_format(self):
        """(format, ell_width): 0 dense blocks, 1 orbital-row ELL, 2 sparse
        blocks staged in shared memory."""
        f, k = C.c_int(), C.c_int()
        check(lib.kpm_batch_format(self._b, C.byref(f), C.byref(k)))
        return f.value, k.value

    def work_order(self):
        """'partition' (the vector groups of a row partition side by side)
        or 'group' (all partitions of one vector group side by side)."""
        g = C.c_int()
        check(lib.kpm_batch_order(self._b, C.byref(g)))
        return 'group' if g.value else 'partition'

    def close(self):
        if getattr(self, '_b', None):
            lib.kpm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()


class Mlp:
    """Multilayer perceptron on the device (kpm_mlp_* C ABI)."""

    def __init__(self, widths, max_batch=4096, seed=0):
        self.widths = [int(w) for w in widths]
        w = np.ascontiguousarray(self.widths, dtype=np.int32)
        m = C.c_void_p()
        check(lib.kpm_mlp_create(len(w) - 1, ptr(w), int(max_batch),
                                 C.c_uint64(int(seed) & (2**64 - 1)),
                                 C.byref(m)))
        self._m = m
        self.max_batch = int(max_batch)
        n = C.c_int64()
        check(lib.kpm_mlp_num_params(m, C.byref(n)))
        self.num_params = n.value

    def get_params(self):
        out = np.empty(self.num_params, dtype=np.float32)
        check(lib.kpm_mlp_get_params(self._m, ptr(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (self.num_params,):
            raise ValueError('expected %d parameters' % self.num_params)
        check(lib.kpm_mlp_set_params(self._m, ptr(p)))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], self.widths[-1]), dtype=np.float32)
        check(lib.kpm_mlp_forward(self._m, ptr(x), x.shape[0], ptr(y)))
        return y

    def gradients(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.num_params, dtype=np.float32)
        loss = C.c_double()
        check(lib.kpm_mlp_gradients(self._m, ptr(x), ptr(y), x.shape[0],
                                    ptr(g), C.byref(loss)))
        return g, loss.value

    def train(self, x, y, batch, epochs, lr, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_double()
        check(lib.kpm_mlp_train(self._m, ptr(x), ptr(y), x.shape[0],
                                int(batch), int(epochs), float(lr),
                                C.c_uint64(int(seed) & (2**64 - 1)),
                                C.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, '_m', None):
            lib.kpm_mlp_destroy(self._m)
            self._m = None

    def __del__(self):
        self.close()
