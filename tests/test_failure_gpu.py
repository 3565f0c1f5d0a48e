"""Failure detection on the GPU without a fault: the bounded mbarrier waits
of the tensor-core kernels.  With a 1 ms wait limit and the test switch
that makes their TMA producers issue no loads, the MMA thread's wait runs
out; the kernel records the expiry, waits for nothing in flight, releases
its tensor memory and returns, and the call reports KPM_ETIMEOUT.  The same
handle then computes the correct result, so the CUDA context stayed
usable."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_tensor_core_wait_expiry_reports_timeout():
    from kwant_gb300 import _lib, kpm, lattices
    if _lib.device_count() == 0:
        pytest.fail('no CUDA device: the GPU tests need a GB300')
    syst = lattices.rashba_square(10, seed=3)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    pos = syst.orbital_positions()
    vx = kpm._velocity(ham, None, 'x', pos)
    vy = kpm._velocity(ham, None, 'y', pos)
    n = ham.shape[0]
    vecs = np.exp(2j * np.pi * np.random.RandomState(2).random_sample((3, n)))
    g = float(np.max(np.asarray(abs(ham).sum(axis=1))))
    a, b = kpm._rescale_ab(-g, g, 0.05)
    _a = a * (1 - 0.05 / 2)
    a2, b2 = kpm._rescale_ab(b - _a, b + _a, 0.05)
    h = _lib.Handle(ham, a, b, _lib.PREC_MIXED)
    M = 32
    ref = _lib.correlator_moments(h, a2, b2, vx, vy, vecs, M, gemm=3)
    try:
        _lib.debug_set(_lib.DEBUG_WAIT_NS, 1000000)
        _lib.debug_set(_lib.DEBUG_STALL_TMA, 1)
        with pytest.raises(_lib.KPMError, match='bounded wait expired'):
            _lib.correlator_moments(h, a2, b2, vx, vy, vecs, M, gemm=1)
    finally:
        _lib.debug_set(_lib.DEBUG_STALL_TMA, 0)
        _lib.debug_set(_lib.DEBUG_WAIT_NS, 2000000000)
    got = _lib.correlator_moments(h, a2, b2, vx, vy, vecs, M, gemm=1)
    assert _rel(got, ref) < 1e-5
    h.close()


def test_debug_keys_checked():
    from kwant_gb300 import _lib
    with pytest.raises(ValueError):
        _lib.debug_set(99, 1)
    with pytest.raises(ValueError):
        _lib.debug_set(_lib.DEBUG_WAIT_NS, 0)
