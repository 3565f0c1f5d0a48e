"""Loading helpers for the golden fixtures in tests/golden/."""

import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    with np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


def csr(g, prefix=''):
    return sp.csr_matrix((g[prefix + 'H_data'], g[prefix + 'H_indices'],
                          g[prefix + 'H_indptr']),
                         shape=tuple(g[prefix + 'H_shape']))


def ref_vectors(seed, n, count, orbs=None):
    """The reference's vector stream for rng=seed: _v0, then one block per
    vector (kwant/kpm.py:201-203, :946-951)."""
    rng = np.random.RandomState(int(seed))
    v0 = np.exp(2j * np.pi * rng.random_sample(n))
    vecs = np.zeros((count, n), dtype=complex)
    idx = np.arange(n) if orbs is None else np.asarray(orbs)
    for r in range(count):
        vecs[r, idx] = np.exp(2j * np.pi * rng.random_sample(len(idx)))
    return v0, vecs
