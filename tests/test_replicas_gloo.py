"""The N > 1 host path on CPU: two gloo ranks combine per-vector moments
and take the slowest rank's time, as bench.py --gpus N does between GPUs;
the moments are those of one run over the union of the ranks' vectors
(checked against the oracle)."""

import os
import socket

import numpy as np
import scipy.sparse as sp

from oracle import kpm_oracle as ko


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _ham():
    rng = np.random.RandomState(0)
    a = sp.random(30, 30, density=0.2, random_state=rng) * (1 + 1j)
    return sp.csr_matrix(a + a.conj().T)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from kwant_gb300 import replicas
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        ham = _ham()
        rng = np.random.RandomState(replicas.replica_seed(10, rank))
        R = 2 + rank                        # uneven vector counts
        vecs = np.exp(2j * np.pi * rng.random_sample((R, 30)))
        local = np.array([ko.moments_dos(ham, 8.0, 0.0, v, 12)[0]
                          for v in vecs])
        allm = replicas.gather_moments(local)
        tmax = replicas.max_over_ranks(1.0 + rank)
        out.put((rank, allm, tmax))
    finally:
        dist.destroy_process_group()


def test_two_rank_combination():
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda r: r[0])
    ham = _ham()
    ref = []
    for rank in range(2):
        rng = np.random.RandomState(10 + rank)
        vecs = np.exp(2j * np.pi * rng.random_sample((2 + rank, 30)))
        ref += [ko.moments_dos(ham, 8.0, 0.0, v, 12)[0] for v in vecs]
    ref = np.array(ref)
    for rank, allm, tmax in res:
        assert allm.shape == (5, 12)
        assert np.array_equal(allm, ref)
        assert tmax == 2.0
