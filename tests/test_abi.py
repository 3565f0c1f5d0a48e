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
