"""Batched multi-system KPM (BSR4, one launch per step for all systems,
CUDA-graph replay) against the CPU oracle."""

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


def _host_wilson_dirac(L, m, W, seed):
    """Host CSR of the Wilson-Dirac model with the device generator's
    disorder (kwant_gb300.lattices conventions)."""
    from kwant_gb300 import lattices, batch
    syst = lattices.wilson_dirac_cubic(L, m=m, W=0.0)
    H = syst.hamiltonian_submatrix(sparse=True).tocsr()
    w = batch.wilson_dirac_disorder(seed, L, W)
    return (H + sp.diags(np.repeat(w, 4))).tocsr()


def _gershgorin(H):
    g = float(np.max(np.asarray(abs(H).sum(axis=1))))
    return -g, g


def _oracle_mean(H, a, b, vecs, M):
    mom = [ko.moments_dos(H, a, b, v.astype(complex), M)[0] for v in vecs]
    return np.mean(np.array(mom), axis=0)


def test_batch_matches_oracle_uneven_sizes():
    from kwant_gb300 import batch
    R, M, seed = 8, 40, 11
    mats = [_host_wilson_dirac(3, 1.5, 1.0, 7), _host_wilson_dirac(5, 1.5, 3.0, 8),
            _host_wilson_dirac(4, 1.0, 0.5, 9)]
    bd = batch.BatchedDOS(R, M, seed=seed)
    for H in mats:
        bd.add_matrix(H, _gershgorin(H))
    mom = bd.moments()
    assert mom.shape == (3, M)
    for s, H in enumerate(mats):
        a, b = bd.scales[s]
        vecs = batch.random_phase_vectors(seed, s, R, H.shape[0])
        ref = _oracle_mean(H, a, b, vecs, M)
        err = np.max(np.abs(mom[s] - ref)) / np.max(np.abs(ref))
        assert err < 1e-5, (s, err)
    # graph replay is deterministic
    assert np.array_equal(bd.moments(), mom)
    ms, nodes, vpl = bd.stats()
    assert ms > 0 and nodes >= M and vpl in (1, 2)
    en, rho = bd.densities(mom)
    assert rho.shape == (3, 2 * M) and np.all(np.isfinite(rho))


def test_batch_mixed_matches_oracle_and_single_vectors():
    """precision='mixed' runs every system through the compensated step
    with the starting vectors of the 'single' batch (the device stream of
    random_phase_vectors): the moments match the oracle on those vectors,
    a rerun repeats them bit for bit, and wilson_dirac_matrix is the host
    twin of the device-generated system."""
    from kwant_gb300 import batch
    R, M, seed = 8, 40, 11
    mats = [_host_wilson_dirac(3, 1.5, 1.0, 7), _host_wilson_dirac(5, 1.5, 3.0, 8)]
    bd = batch.BatchedDOS(R, M, seed=seed, precision='mixed')
    for H in mats:
        bd.add_matrix(H, _gershgorin(H))
    bd.add_wilson_dirac(4, m=1.5, W=0.5, seed=9)
    mats.append(batch.wilson_dirac_matrix(4, 1.5, 0.5, 9))
    assert np.array_equal(mats[-1].toarray(),
                          _host_wilson_dirac(4, 1.5, 0.5, 9).toarray())
    mom = bd.moments()
    assert mom.shape == (3, M)
    for s, H in enumerate(mats):
        a, b = bd.scales[s]
        vecs = batch.random_phase_vectors(seed, s, R, H.shape[0])
        ref = _oracle_mean(H, a, b, vecs, M)
        err = np.max(np.abs(mom[s] - ref)) / np.max(np.abs(ref))
        # complex64 values of 2H/a: a consistent ~6e-8 perturbation of H
        assert err < 2e-6, (s, err)
    assert np.array_equal(bd.moments(), mom)     # rerun: same vectors
    ms, launches, _ = bd.stats()
    assert ms > 0 and launches >= 3 * M // 2
    assert bd.step_format() == (3, 0)
    bd.close()
    with pytest.raises(ValueError):
        batch.BatchedDOS(4, 24, precision='fp64')


def test_device_generated_wilson_dirac_equals_host_matrix():
    from kwant_gb300 import batch
    R, M, seed = 4, 24, 5
    L, m, W, dseed = 5, 1.5, 2.0, 3
    H = _host_wilson_dirac(L, m, W, dseed)
    bounds = _gershgorin(H)
    a = batch.BatchedDOS(R, M, seed=seed)
    a.add_wilson_dirac(L, m=m, W=W, seed=dseed, bounds=bounds)
    b = batch.BatchedDOS(R, M, seed=seed)
    b.add_matrix(H, bounds)
    ma, mb = a.moments(), b.moments()
    assert np.max(np.abs(ma - mb)) / np.max(np.abs(mb)) < 1e-6


def test_batch_rejects_bad_input():
    from kwant_gb300 import batch
    with pytest.raises(ValueError):
        batch.BatchedDOS(4, 25)            # odd number of moments
    bd = batch.BatchedDOS(4, 24)
    wide = sp.random(40, 40, density=1.0, format='csr') + 0j
    with pytest.raises(ValueError):
        bd.add_matrix(wide + wide.conj().T, (-50.0, 50.0))  # > 8 blocks/row


def test_sparse_blocks_run_as_orbital_ell(monkeypatch):
    """Wilson-Dirac blocks are half empty: the batch can convert them to an
    orbital-row ELL (13 entries per row, width 16) on the device; forced
    either way, the two step kernels agree with each other and with the
    oracle (the autotuner picks the faster one)."""
    from kwant_gb300 import batch
    R, M, seed = 8, 40, 3
    mats = [_host_wilson_dirac(4, 1.5, 2.0, 5), _host_wilson_dirac(3, 1.5, 0.7, 6)]

    def run():
        bd = batch.BatchedDOS(R, M, seed=seed)
        for H in mats:
            bd.add_matrix(H, _gershgorin(H))
        bd.add_wilson_dirac(5, m=1.5, W=1.0, seed=9,
                            bounds=_gershgorin(_host_wilson_dirac(5, 1.5, 1.0, 9)))
        return bd, bd.moments()

    monkeypatch.setenv('KPM_BATCH_FORMAT', 'ell')
    bd_ell, m_ell = run()
    assert bd_ell.step_format() == (1, 16)
    monkeypatch.setenv('KPM_BATCH_FORMAT', 'sparse')
    bd_sb, m_sb = run()
    assert bd_sb.step_format()[0] == 2
    monkeypatch.setenv('KPM_BATCH_FORMAT', 'bsr')
    bd_bsr, m_bsr = run()
    assert bd_bsr.step_format() == (0, 0)
    assert np.max(np.abs(m_ell - m_bsr)) <= 1e-6 * np.max(np.abs(m_bsr))
    assert np.max(np.abs(m_sb - m_bsr)) <= 1e-6 * np.max(np.abs(m_bsr))
    for s, H in enumerate(mats):
        a, b = bd_ell.scales[s]
        vecs = batch.random_phase_vectors(seed, s, R, H.shape[0])
        ref = _oracle_mean(H, a, b, vecs, M)
        assert np.max(np.abs(m_ell[s] - ref)) / np.max(np.abs(ref)) < 1e-5
        assert np.max(np.abs(m_sb[s] - ref)) / np.max(np.abs(ref)) < 1e-5


def test_work_orders_give_identical_moments(monkeypatch):
    """The two work orders of the BSR and ELL step kernels (a partition's
    vector groups side by side, or all partitions of a vector group side by
    side) change only which block computes what when: the moments are
    bit-identical, and the batch reports the order it ran."""
    from kwant_gb300 import batch
    R, M, seed = 64, 24, 4
    mats = [_host_wilson_dirac(6, 1.5, 1.5, 2), _host_wilson_dirac(4, 1.5, 0.3, 3)]

    def run(fmt, order):
        monkeypatch.setenv('KPM_BATCH_FORMAT', fmt)
        monkeypatch.setenv('KPM_BATCH_ORDER', order)
        bd = batch.BatchedDOS(R, M, seed=seed)
        for H in mats:
            bd.add_matrix(H, _gershgorin(H))
        mom = bd.moments()
        assert bd.work_order() == order
        return mom

    for fmt in ('bsr', 'ell'):
        assert np.array_equal(run(fmt, 'partition'), run(fmt, 'group')), fmt


def test_dense_blocks_stay_bsr():
    from kwant_gb300 import batch
    rng = np.random.RandomState(0)
    n = 32                # 8 block rows, 5 dense 4x4 blocks: 20 per row
    A = sp.random(n, n, density=1.0, random_state=rng, dtype=float)
    mask = sp.kron(sp.diags([1.0] * 5, [-2, -1, 0, 1, 2], shape=(8, 8)),
                   np.ones((4, 4)))
    H = A.multiply(mask) * (1 + 0.5j)
    H = (H + H.conj().T).tocsr()
    assert np.diff(H.indptr).max() == 20
    R, M = 4, 16
    bd = batch.BatchedDOS(R, M, seed=1)
    bd.add_matrix(H, _gershgorin(H))
    mom = bd.moments()
    assert bd.step_format()[0] == 0
    a, b = bd.scales[0]
    vecs = batch.random_phase_vectors(1, 0, R, n)
    ref = _oracle_mean(H, a, b, vecs, M)
    assert np.max(np.abs(mom[0] - ref)) / np.max(np.abs(ref)) < 1e-5
