"""The bounds-checked debug library (-DKPM_CHECK: every gathered column
index of the Chebyshev step kernels is validated on the device) runs the
DOS path and reproduces the reference's moments: the checks change no
result and find no index out of range.  Runs in a fresh process that loads
the checked build through KWANT_GB300_LIB."""

import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import numpy as np, sys
sys.path[:0] = [%(root)r, %(tests)r]
from golden_io import load, csr, ref_vectors
from kwant_gb300 import _lib, kpm
assert _lib.build_checks()
g = load('square100')
ham = csr(g)
a, b = kpm._rescale_ab(g['lmin'], g['lmax'], 0.05)
_, vecs = ref_vectors(g['seed'], ham.shape[0], 10)
ref = g['moments_list']
for prec, tol in ((_lib.PREC_FP64, 1e-12), (_lib.PREC_MIXED, 1e-6),
                  (_lib.PREC_SINGLE, 1e-5)):
    h = _lib.Handle(ham, a, b, prec, reorder=prec != _lib.PREC_FP64)
    blk = _lib.Block(h, vecs, keep_a0=True)
    mom = blk.dos_moments(0, 100)
    err = np.max(np.abs(mom - ref)) / np.max(np.abs(ref))
    assert err < tol, (prec, err)
    blk.close(); h.close()
print('ok')
'''


def test_checked_build_reproduces_reference_moments():
    from kwant_gb300 import build
    checked = build.build(variant='check')
    env = dict(os.environ, KWANT_GB300_LIB=checked)
    code = SCRIPT % {'root': ROOT, 'tests': os.path.join(ROOT, 'tests')}
    out = subprocess.run([sys.executable, '-c', code], cwd=ROOT, env=env,
                         capture_output=True, text=True, timeout=900)
    assert out.returncode == 0 and 'ok' in out.stdout, out.stderr[-3000:]
