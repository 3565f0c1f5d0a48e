"""Checkpoint / resume of SpectralDensity (save -> load in a new object):
resuming must be bit-identical to continuing the original object, for the
DOS and for an operator, in both precisions, and add_vectors must continue
the same random-vector stream."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('with_op', [False, True])
def test_save_load_resumes_exactly(tmp_path, precision, with_op):
    from kwant_gb300 import kpm, lattices, operator
    syst = lattices.square(12, seed=4)
    H = syst.hamiltonian_submatrix(sparse=True)
    op = operator.Density(syst, where=[0, 5, 17]) if with_op else None
    kw = dict(params=None, operator=op, num_moments=30, num_vectors=4,
              rng=7, precision=precision)
    sd = kpm.SpectralDensity(syst, **kw)
    f = tmp_path / 'ckpt.npz'
    sd.save(f)
    sd2 = kpm.SpectralDensity.load(f, syst, operator=op)
    assert np.array_equal(sd2.densities, sd.densities)
    assert np.array_equal(sd2.energies, sd.energies)
    for s in (sd, sd2):
        s.add_moments(21)
    assert sd2.num_moments == sd.num_moments == 51
    assert np.array_equal(np.array(sd2._moments_list),
                          np.array(sd._moments_list))
    assert np.array_equal(sd2.densities, sd.densities)
    for s in (sd, sd2):
        s.add_vectors(3)
    assert np.array_equal(np.array(sd2._moments_list),
                          np.array(sd._moments_list))
    # and the same as a fresh run with all moments and vectors at once
    fresh = kpm.SpectralDensity(syst, **dict(kw, num_moments=51,
                                             num_vectors=7))
    assert np.allclose(fresh.densities, sd2.densities, rtol=1e-12,
                       atol=1e-12 * np.abs(fresh.densities).max())
    with pytest.raises(ValueError):
        kpm.SpectralDensity.load(f, lattices.square(11, seed=4))


def test_load_continues_a_user_vector_list(tmp_path):
    """A checkpoint of a run on user-supplied vectors, loaded with the same
    list: add_vectors continues with the list's next vectors (the saved
    ones are skipped), as an uninterrupted run does."""
    from kwant_gb300 import kpm, lattices
    syst = lattices.square(10, seed=2)
    n = syst.hamiltonian_submatrix(sparse=True).shape[0]
    vecs = list(np.exp(2j * np.pi * np.random.RandomState(4)
                       .random_sample((6, n))))
    kw = dict(num_moments=24, bounds=(-4.6, 4.6))
    sd = kpm.SpectralDensity(syst, vector_factory=vecs, num_vectors=3, **kw)
    f = tmp_path / 'ckpt.npz'
    sd.save(f)
    sd2 = kpm.SpectralDensity.load(f, syst, vector_factory=vecs)
    sd2.add_vectors(3)
    full = kpm.SpectralDensity(syst, vector_factory=vecs, num_vectors=6, **kw)
    assert np.array_equal(np.array(sd2._moments_list),
                          np.array(full._moments_list))


def test_checkpoint_needs_accumulated_vectors(tmp_path):
    from kwant_gb300 import kpm, lattices
    syst = lattices.square(8, seed=1)
    sd = kpm.SpectralDensity(syst, num_moments=10, num_vectors=2, rng=0,
                             accumulate_vectors=False)
    with pytest.raises(ValueError):
        sd.save(tmp_path / 'x.npz')
