"""Host side of the starting vectors, on the CPU: RandomVectors draws the
reference's stream (kwant/kpm.py:932-951: exp(2 pi i u), u from
RandomState.random_sample, one draw per vector), bit for bit, including the
chunked multi-threaded evaluation of long vectors; the rows are stacked
into one array exactly as np.array stacks them."""

import numpy as np
import pytest
import scipy.sparse as sp

from kwant_gb300 import kpm


def _reference_vectors(seed, n, count):
    rng = np.random.RandomState(seed)
    return [np.exp(2j * np.pi * rng.random_sample(n)) for _ in range(count)]


@pytest.mark.parametrize('n', [1000, 1_200_000])   # the second is chunked
def test_random_vectors_bit_identical_to_reference_stream(n):
    ham = sp.identity(n, dtype=complex, format='csr')
    gen = kpm.RandomVectors(ham, rng=7)
    ref = _reference_vectors(7, n, 3)
    for r in ref:
        assert np.array_equal(next(gen), r)


def test_random_vectors_where_subset():
    n = 50
    ham = sp.identity(n, dtype=complex, format='csr')
    where = [3, 10, 11, 40]
    gen = kpm.RandomVectors(ham, where=where, rng=2)
    rng = np.random.RandomState(2)
    for _ in range(2):
        v = next(gen)
        want = np.zeros(n, complex)
        want[where] = np.exp(2j * np.pi * rng.random_sample(len(where)))
        assert np.array_equal(v, want)


@pytest.mark.parametrize('shape', [(3, 10), (4, 1 << 20)])
def test_stack_vectors_equals_np_array(shape):
    rng = np.random.RandomState(0)
    rows = [rng.random_sample(shape[1]) + 1j * rng.random_sample(shape[1])
            for _ in range(shape[0])]
    got = kpm._stack_vectors(iter(rows))
    assert got.dtype == complex and got.shape == shape
    assert np.array_equal(got, np.array(rows))


def test_stack_vectors_ragged_raises():
    with pytest.raises(ValueError):
        kpm._stack_vectors([np.ones(3), np.ones(4)])
