"""kpm_dos_moments_noalloc: the DOS recursion for callers that cannot let the
library allocate device memory (frameworks that own every device byte
through their own arena, services with a fixed device-memory budget).

The test plays such a caller: it allocates every buffer itself (with torch)
and passes device pointers through the C ABI; the result must match the
regular, allocating entry point (kpm_block_dos_moments) within the FP64
parity tolerance of the other tests, on two calls in a row (the second call
runs over the scratch the first one left behind); in FP64 it must also
match the reference's own moments (the square100 fixture).  In mixed
precision this entry point runs the plain complex64 recursion, so it is
compared with a handle in that form (KPM_FLAG_PLAIN_C64): the two compute
the same Chebyshev vectors with different step kernels (CSR here, ELL
there) whose FP32 dot-product partials group the rows differently, so they
agree to FP32 partial-sum rounding (1e-8).  This file is collected last so
that a failure here does not stop the rest of the GPU suite.
"""

import ctypes as C

import numpy as np
import pytest

from golden_io import load, csr, ref_vectors

pytestmark = pytest.mark.gpu

TOL = {'fp64': 1e-12, 'mixed': 1e-8}


class DeviceCsr(C.Structure):
    _fields_ = [('rows', C.c_int64), ('nnz', C.c_int64),
                ('indptr', C.c_void_p), ('indices', C.c_void_p),
                ('data', C.c_void_p)]


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_noalloc_matches_allocating_entry_point(precision):
    torch = pytest.importorskip('torch')
    from kwant_gb300 import _lib, kpm
    assert torch.cuda.is_available(), 'needs a CUDA device'

    g = load('square100')
    ham = csr(g)
    n = ham.shape[0]
    a, b = kpm._rescale_ab(g['lmin'], g['lmax'], 0.05)
    R, M = 10, 101                      # odd M: exercises the norm-only tail
    _, vecs = ref_vectors(g['seed'], n, R)
    mixed = precision == 'mixed'
    prec = _lib.PREC_MIXED if mixed else _lib.PREC_FP64

    # the existing, allocating entry point (plain complex64 form in mixed
    # precision, the arithmetic of this entry point)
    h = _lib.Handle(ham, a, b, _lib.PREC_SINGLE if mixed else prec)
    blk = _lib.Block(h, vecs, keep_a0=True)
    expected = blk.dos_moments(0, M)
    blk.close()
    h.close()

    # caller-owned device buffers
    dev = torch.device('cuda')
    G = 32 if mixed else 16
    Rpad = -(-R // G) * G
    ctype = np.complex64 if mixed else np.complex128
    indptr = torch.from_numpy(ham.indptr.astype(np.int32)).to(dev)
    indices = torch.from_numpy(ham.indices.astype(np.int32)).to(dev)
    if mixed:
        vals = (ham.data * (2.0 / a)).astype(np.complex64)
    else:
        vals = ham.data.astype(np.complex128)
    vals_d = torch.from_numpy(vals.view(np.float32 if mixed else
                                        np.float64).copy()).to(dev)
    host_vecs = np.zeros((n, Rpad), dtype=ctype)
    host_vecs[:, :R] = vecs.T
    vecs_d = torch.from_numpy(host_vecs.view(np.float32 if mixed else
                                             np.float64).copy()).to(dev)
    elem = 8 if mixed else 16
    work = torch.empty(2 * n * Rpad * elem, dtype=torch.uint8, device=dev)
    moments = torch.empty(M * Rpad * 2, dtype=torch.float64, device=dev)
    desc = DeviceCsr(n, ham.nnz, indptr.data_ptr(), indices.data_ptr(),
                     vals_d.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream

    for call in range(2):
        moments.fill_(float('nan'))
        st = _lib.lib.kpm_dos_moments_noalloc(
            C.byref(desc), C.c_double(a), C.c_double(b), prec,
            C.c_void_p(vecs_d.data_ptr()), R, M, C.c_void_p(work.data_ptr()),
            C.c_void_p(moments.data_ptr()), C.c_void_p(stream))
        _lib.check(st)
        torch.cuda.synchronize()
        got = moments.cpu().numpy().view(np.complex128).reshape(M, Rpad)
        got = got[:, :R].T
        err = np.max(np.abs(got - expected)) / np.max(np.abs(expected))
        assert err < TOL[precision], (call, err)
        # against the reference's own moments (golden fixture): FP64 to
        # rounding; the complex64 recursion within 1e-5 of the largest
        # moment (a numpy complex64 recursion of these vectors: 1e-7)
        ref = g['moments_list']
        err = np.max(np.abs(got[:, :ref.shape[1]] - ref)) / \
            np.max(np.abs(ref))
        assert err < (1e-5 if mixed else TOL[precision]), (call, err)


def test_noalloc_rejects_oversized_requests():
    torch = pytest.importorskip('torch')
    from kwant_gb300 import _lib
    assert torch.cuda.is_available(), 'needs a CUDA device'
    n = 1 << 16
    desc = DeviceCsr(n, 0, 1, 1, 0)   # never dereferenced: rejected first
    with pytest.raises(ValueError, match='scratch'):
        _lib.check(_lib.lib.kpm_dos_moments_noalloc(
            C.byref(desc), C.c_double(1.0), C.c_double(0.0), _lib.PREC_FP64,
            C.c_void_p(1), 4096, 10, C.c_void_p(1), C.c_void_p(1),
            C.c_void_p(0)))
