"""The C-ABI library loads and exports exactly the symbols the header
declares.  No compute calls: this runs without a GPU."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'kwant_gb300.h')


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r'KPM_API\s+int\s+(kpm_\w+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib_path():
    from kwant_gb300 import build
    return build.build()


def test_header_declares_api():
    names = _declared()
    assert 'kpm_create' in names and 'kpm_block_dos_moments' in names
    assert len(names) >= 20


def test_library_loads_and_exports_every_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in _declared():
        assert hasattr(lib, name), name


def test_no_extra_exports(lib_path):
    out = subprocess.run(['nm', '-D', '--defined-only', lib_path],
                         capture_output=True, text=True, check=True).stdout
    exported = sorted(l.split()[-1] for l in out.splitlines()
                      if ' T ' in l and l.split()[-1].startswith('kpm_'))
    assert exported == _declared()


def test_python_binding_covers_every_symbol():
    from kwant_gb300 import _lib
    for name in _declared():
        fn = getattr(_lib.lib, name)
        assert fn.restype is ctypes.c_int, name


def test_device_count_without_gpu_is_graceful():
    from kwant_gb300 import _lib
    n = _lib.device_count()
    assert n >= 0


def test_argument_checks_and_missing_device_fail_cleanly():
    """Invalid arguments are rejected before any device work, and without a
    usable device every computing entry point returns KPM_ECUDA with a
    message (there is no CPU fallback); nothing crashes."""
    import numpy as np
    from kwant_gb300 import _lib
    lib = _lib.lib
    P = ctypes.c_void_p
    out = P()
    # null / invalid arguments: KPM_EINVAL
    assert lib.kpm_create(None, 1.0, 0.0, 0, ctypes.byref(out)) == -1
    assert lib.kpm_family_point(None, 0.0, 0.0, 0.0) == -1
    assert lib.kpm_chebval(0, 1, None, 0, None, None) == -1
    w = np.array([3, 100, 32], np.int32)            # hidden width % 32 != 0
    assert lib.kpm_mlp_create(2, w.ctypes.data_as(P), 64, 0,
                              ctypes.byref(out)) == -1
    assert lib.kpm_batch_create(4, 25, 0, ctypes.byref(out)) == -1  # odd M
    assert lib.kpm_block_restore(None, 0, 0, None, None, None) == -1
    if _lib.device_count() == 0:
        m = np.eye(3, dtype=complex)
        import scipy.sparse as sp
        csr = _lib.Csr(sp.csr_matrix(m + np.diag([0, 1, 2])))
        st = lib.kpm_create(csr.ref(), 2.0, 0.0, 0, ctypes.byref(out))
        assert st == -2                                  # KPM_ECUDA
        assert 'CUDA' in _lib.last_error()
        assert lib.kpm_batch_create(4, 24, 0, ctypes.byref(out)) == -2


def test_batch_arguments_checked_on_the_host():
    """BatchedDOS rejects an unknown precision and an odd moment count
    before any device work, in both precisions."""
    import pytest
    from kwant_gb300 import batch
    with pytest.raises(ValueError):
        batch.BatchedDOS(4, 24, precision='fp64')
    for prec in ('single', 'mixed'):
        with pytest.raises(ValueError):
            batch.BatchedDOS(4, 25, precision=prec)
    bd = batch.BatchedDOS(4, 24, precision='mixed')   # nothing on the device
    assert bd.stats()[0] == 0.0 and bd.step_format() == (3, 0)
    H = batch.wilson_dirac_matrix(3, 1.5, 1.0, 7)
    assert H.shape == (108, 108) and abs(H - H.conj().T).max() == 0
    with pytest.raises(ValueError):
        bd.add_matrix(H[:107, :107], (-10.0, 10.0))    # not 4-orbital


def _query_checks(lib_file):
    """kpm_build_checks of a library, in a fresh process that loads it
    through the package (KWANT_GB300_LIB)."""
    env = dict(os.environ, KWANT_GB300_LIB=lib_file)
    out = subprocess.run(
        ['python', '-c', 'from kwant_gb300 import _lib; '
         'print(int(_lib.build_checks()))'],
        cwd=ROOT, env=env, capture_output=True, text=True, check=True)
    return int(out.stdout.strip())


def test_bounds_checked_build(lib_path):
    """The -DKPM_CHECK debug build (in-kernel index validation) compiles,
    links, exports the same symbols and reports itself; the default
    library does not check."""
    from kwant_gb300 import build
    checked = build.build(variant='check')
    assert os.path.abspath(checked) != os.path.abspath(lib_path)
    lib = ctypes.CDLL(checked)
    for name in _declared():
        assert hasattr(lib, name), name
    assert _query_checks(checked) == 1
    assert _query_checks(lib_path) == 0
