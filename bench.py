"""Benchmark of the KPM hot path: KPM nnz*vec*moment/s.

Workload (default): the honeycomb (graphene) DOS workload -- 1000 x 1000
unit cells (2e6 orbitals), hopping t = 1 with a Peierls phase of 1/1000 flux
quanta per hexagon, Anderson disorder W = 0.5 (seed 0), R = 64 random-phase
vectors (rng seed 1, the reference's stream), M = 2000 moments, DOS
(operator=None), mixed precision (complex64 recursion, FP64 accumulation).
Synthetic data built by kwant_gb300.lattices; the vector blocks (1 GB each)
are larger than L2, so no L2 flush is needed between steps.

A "step" is one complete moment computation (R vectors x M moments) of the
workload.  value = nnz * R * M / (device time per step), with the Hamiltonian
and vectors resident in HBM.  e2e is the same metric through the C ABI's
one-shot kpm_dos() with pinned host buffers: Hamiltonian upload, vector
upload, recursion, device reconstruction and result download every step.

--impl reference times the reference's CPU algorithm (the oracle port of
kwant.kpm: scipy CSR matvec + vdot, one vector at a time) on the host cores,
one spawned process per core over disjoint vectors, on a bounded sample.
"""

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'KPM nnz*vec*moment/s'
UNIT = 'nnz*vec*moment/s'


# ---------------------------------------------------------------- workload
def make_workload(cells, vectors, seed_dis=0, seed_vec=1):
    from kwant_gb300 import lattices
    syst = lattices.honeycomb(cells, t=1.0, flux=1.0 / 1000, W=0.5,
                              seed=seed_dis)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    n = ham.shape[0]
    rng = np.random.RandomState(seed_vec)
    v0 = np.exp(2j * np.pi * rng.random_sample(n))   # the reference's _v0
    vecs = np.empty((vectors, n), dtype=np.complex128)
    for r in range(vectors):
        vecs[r] = np.exp(2j * np.pi * rng.random_sample(n))
    return ham, v0, vecs


VEC_BYTES = {'mixed': 12, 'single': 8, 'fp64': 16}


def step_bytes(nnz, n, R, precision):
    """Algorithmic HBM bytes of one Chebyshev step over R vectors:
    values + column indices + row pointers + read alpha_n, read alpha_{n-1},
    write alpha_{n+1}.  Vector elements: complex64 plus a bfloat16 x 2
    correction (12 B, 'mixed'), complex64 (8 B, 'single') or complex128
    (16 B); values complex64 (8 B) or complex128 (16 B)."""
    sv = 16 if precision == 'fp64' else 8
    return nnz * sv + 4 * nnz + 4 * (n + 1) + 3 * n * R * VEC_BYTES[precision]


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ('clocks.sm,clocks.max.sm,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index),
                 '--query-gpu=' + self.FIELDS, '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for line in self.lines:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower() == 'active':
                    reasons.add(nm)
        if not sm:
            return None
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ------------------------------------------------------------ CPU baseline
_W = {}


def _cpu_init(path, a, b, where=None):
    import scipy.sparse as sp
    d = np.load(path)
    _W['ham'] = sp.csr_matrix((d['data'], d['indices'], d['indptr']),
                              shape=tuple(d['shape']))
    _W['a'], _W['b'] = a, b
    _W['where'] = where


def _cpu_task(args):
    from oracle import kpm_oracle as ko
    vec, M = args
    t0 = time.perf_counter()
    if _W['where'] is None:
        ko.moments_dos(_W['ham'], _W['a'], _W['b'], vec, M)
    else:
        # Density (identity onsite) on one-orbital sites, the operator path
        # (kwant/kpm.py:478-484); density_matels' products for norbs = 1,
        # vectorised over the sites
        n = _W['ham'].shape[0]
        start, _ = ko.site_orbitals([(0, 1, 0), (n, 0, n)], _W['where'])
        start = np.asarray(start)

        def op(bra, ket):
            return np.conj(bra[start]) * ket[start]
        ko.moments_operator(_W['ham'], _W['a'], _W['b'], vec, M, op)
    return time.perf_counter() - t0


def _oracle_task(args):
    """The oracle's FP64 moments of one vector (the checker, untimed)."""
    from oracle import kpm_oracle as ko
    vec, M = args
    return np.array(ko.moments_dos(_W['ham'], _W['a'], _W['b'], vec, M)[0])


class CpuBaseline:
    """The oracle port of the reference (one vector at a time, scipy CSR
    matvec + vdot), one spawned process per core over disjoint vectors."""

    def __init__(self, ham, a, b, vecs, procs, where=None):
        self.tmp = tempfile.NamedTemporaryFile(suffix='.npz', delete=False)
        self.tmp.close()
        np.savez(self.tmp.name, data=ham.data, indices=ham.indices,
                 indptr=ham.indptr, shape=np.array(ham.shape))
        self.nnz = ham.nnz
        self.procs = procs
        self.vecs = vecs
        self.pool = _spawn_pool(procs, _cpu_init, (self.tmp.name, a, b,
                                                   where))

    def run(self, M):
        t0 = time.perf_counter()
        jobs = [(self.vecs[r % len(self.vecs)], M) for r in range(self.procs)]
        self.pool.map(_cpu_task, jobs)
        dt = time.perf_counter() - t0
        return self.nnz * self.procs * M / dt, dt

    def oracle_moments(self, vecs, M):
        """(k, M) oracle moments of the given vectors, one process each."""
        return np.array(self.pool.map(_oracle_task, [(v, M) for v in vecs]))

    def close(self):
        self.pool.close()
        self.pool.join()
        os.unlink(self.tmp.name)


def _spawn_pool(procs, init, initargs):
    """A spawned process pool whose workers run single-threaded BLAS /
    OpenMP (one process per core; many processes each with a threaded BLAS
    oversubscribe the cores)."""
    keys = ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS')
    old = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = '1'
    try:
        return mp.get_context('spawn').Pool(procs, initializer=init,
                                            initargs=initargs)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


# ---------------------------------------------------------------- main arms
def dist_setup():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    return world, rank


def run_reference(args):
    world, rank = dist_setup()
    if rank != 0:
        return 0
    ham, v0, vecs = make_workload(args.cells, min(args.vectors, 64))
    # Gershgorin bounds on the host: the reference's ARPACK bounds are not
    # part of the timed moment computation, and this arm runs no GPU code.
    row_abs = np.asarray(abs(ham).sum(axis=1)).ravel()
    hi = float(np.max(row_abs))
    a, b = hi / (1 - 0.05 / 2), 0.0
    procs = args.cpu_procs or os.cpu_count() or 1
    base = CpuBaseline(ham, a, b, vecs, procs)
    try:
        for _ in range(args.warmup):
            base.run(args.ref_moments)
        vals, dts = [], []
        for _ in range(args.steps):
            v, dt = base.run(args.ref_moments)
            vals.append(v)
            dts.append(dt)
    finally:
        base.close()
    value = float(np.median(vals))
    sample = ('%d vectors x %d moments of the %s workload per step, one '
              'spawned process per vector' % (procs, args.ref_moments,
                                               _workload_name(args)))
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT,
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * float(np.median(dts)),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'c128', 'data': 'synthetic',
        'config': {'workload': _workload_name(args), 'nnz': int(ham.nnz),
                   'R': procs, 'M': args.ref_moments},
        'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': procs,
                         'kind': 'port', 'sample': sample,
                         'cpu': _cpu_model()},
        'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))
    return 0


def _cpu_model():
    """The host CPU's model name (from /proc/cpuinfo; Arm cores report no
    model name, then the implementer / part codes), and the machine type."""
    import platform
    name, impl, part = None, None, None
    try:
        with open('/proc/cpuinfo') as f:
            for line in f:
                k, _, v = line.partition(':')
                k, v = k.strip(), v.strip()
                if k == 'model name' and name is None:
                    name = v
                elif k == 'CPU implementer' and impl is None:
                    impl = v
                elif k == 'CPU part' and part is None:
                    part = v
    except OSError:
        pass
    if name is None and impl is not None:
        arm = {'0xd0c': 'Neoverse-N1', '0xd40': 'Neoverse-V1',
               '0xd49': 'Neoverse-N2', '0xd4f': 'Neoverse-V2'}
        name = ('Arm ' + arm[part] if impl == '0x41' and part in arm
                else 'implementer %s part %s' % (impl, part))
    return '%s (%s)' % (name or 'unknown', platform.machine())


def _workload_name(args):
    return ('honeycomb %dx%d cells (%d orbitals), Peierls flux 1/1000, '
            'W=0.5, DOS R=%d M=%d' % (args.cells, args.cells,
                                      2 * args.cells ** 2, args.vectors,
                                      args.moments))


def run_ours(args):
    import torch
    from kwant_gb300 import _lib, kpm

    world, rank = dist_setup()
    if world > 1:
        import torch.distributed as dist
        local = int(os.environ.get('LOCAL_RANK', '0'))
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    dev = torch.cuda.current_device()

    t_setup = time.perf_counter()
    ham, v0, vecs = make_workload(args.cells, args.vectors,
                                  seed_vec=1 + rank)
    n, nnz = ham.shape[0], ham.nnz
    R, M = args.vectors, args.moments
    lo, hi = kpm.spectral_bounds(ham, 0.05, v0, 'lanczos')
    a, b = kpm._rescale_ab(lo, hi, 0.05)
    prec = {'mixed': _lib.PREC_MIXED, 'single': _lib.PREC_SINGLE,
            'fp64': _lib.PREC_FP64}[args.precision]
    csr = _lib.Csr(ham)
    handle = _lib.Handle(csr, a, b, prec,
                         reorder=args.reorder and args.precision != 'fp64')
    block = _lib.Block(handle, vecs, keep_a0=True)
    stream = torch.cuda.ExternalStream(handle.stream())
    setup_s = time.perf_counter() - t_setup

    def one_step():
        block.rewind()
        return block.dos_moments(0, M)

    for _ in range(args.warmup):
        one_step()

    # ---- timed region (device resident) ---------------------------------
    clocks = ClockSampler(dev)
    clocks.start()
    handle.profile(True)
    launches0 = _lib.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    mom = None
    for _ in range(args.steps):
        mom = one_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = _lib.launch_count() - launches0
    n_step, step_ms = handle.profile_read()
    handle.profile(False)
    clk = clocks.stop()
    t_ms = ev0.elapsed_time(ev1)
    if world > 1:
        from kwant_gb300 import replicas
        t_ms = replicas.max_over_ranks(t_ms, device='cuda')
    ms_per_step = t_ms / args.steps
    value = world * nnz * R * M / (ms_per_step / 1e3)

    # ---- roofline of the dominant kernel (the fused step) ----------------
    import json as _json
    peaks = {}
    pk = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(pk):
        peaks = _json.load(open(pk))
    hbm_peak = float(peaks.get('hbm_gbs', 6800.0))
    peak_src = 'measured' if 'hbm_gbs' in peaks else 'fallback'
    B = step_bytes(nnz, n, R, args.precision)
    avg_step_ms = step_ms / max(n_step, 1)
    achieved = B / (avg_step_ms / 1e3) / 1e9
    # DRAM bytes per step launch, ncu dram__bytes_read + dram__bytes_write:
    # 'mixed', a one-pass capture of two step launches of this default
    # workload (1000 x 1000 cells, R = 64): 3.813 + 1.501 GB against 4.712
    # GB algorithmic; 'single', one launch on the 500 x 500-cell case,
    # 774.5 MB against 794.0 MB, scaled by the algorithmic bytes
    traffic = None
    if args.reorder and R == 64:
        if args.precision == 'mixed':
            traffic = B * ((3.813 + 1.501) / 4.712) if args.cells == 1000 \
                else None
        elif args.precision == 'single':
            traffic = B * (774.5 / 794.0)

    # ---- e2e through the C ABI one-shot call (host buffers) ----------------
    e2e = None
    if args.e2e and rank == 0 and args.precision != 'single':
        pin_vec = torch.empty((R, n, 2), dtype=torch.float64,
                              pin_memory=True)
        pin_vec.numpy()[:] = vecs.view(np.float64).reshape(R, n, 2)
        pv = pin_vec.numpy().view(np.complex128).reshape(R, n)
        pins = {}
        for k, arr in (('indptr', csr.indptr), ('indices', csr.indices),
                       ('data', csr.data.view(np.float64))):
            t = torch.empty(arr.shape, dtype={
                np.dtype(np.int32): torch.int32,
                np.dtype(np.float64): torch.float64}[arr.dtype],
                pin_memory=True)
            t.numpy()[:] = arr
            pins[k] = t
        pcsr = _lib.Csr.__new__(_lib.Csr)
        pcsr.shape = csr.shape
        pcsr.indptr = pins['indptr'].numpy()
        pcsr.indices = pins['indices'].numpy()
        pcsr.data = pins['data'].numpy().view(np.complex128)
        pcsr.nnz = csr.nnz
        pcsr.desc = _lib.CsrDesc(n, csr.nnz, _lib.ptr(pcsr.indptr),
                                 _lib.ptr(pcsr.indices), _lib.ptr(pcsr.data))
        out_m = torch.empty((R, M, 2), dtype=torch.float64, pin_memory=True)
        out_g = torch.empty((2 * M, 2), dtype=torch.float64, pin_memory=True)
        out_d = torch.empty((2 * M, 2), dtype=torch.float64, pin_memory=True)
        import ctypes as C

        def e2e_step():
            _lib.check(_lib.lib.kpm_dos(
                C.byref(pcsr.desc), float(a), float(b), prec, _lib.ptr(pv),
                R, M, _lib.KERNEL_JACKSON, C.c_void_p(out_m.data_ptr()),
                C.c_void_p(out_g.data_ptr()), C.c_void_p(out_d.data_ptr())))

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        h2d = csr.indptr.nbytes + csr.indices.nbytes + csr.data.nbytes + \
            vecs.nbytes
        d2h = out_m.numel() * 8 + out_g.numel() * 8 + out_d.numel() * 8
        e2e = {'value': nnz * R * M / (e_ms / 1e3), 'unit': UNIT,
               'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h),
               'ms_per_step': e_ms, 'api': 'kpm_dos (C ABI, pinned host '
               'buffers, handle create + uploads + recursion + device '
               'reconstruction + downloads per step)'}

    # ---- accuracy vs the FP64 path (untimed) -------------------------------
    accuracy = None
    nodes = kpm._chebyshev_nodes(2 * M)

    def dos_k(mm):
        """Densities (mean over the given vectors' moments, Jackson kernel,
        device reconstruction) at the 2M nodes."""
        return _lib.reconstruct(mm[:, :, None], True, False, a,
                                _lib.KERNEL_JACKSON, 4.0, nodes)[1][:, 0]

    mom64 = None
    if args.accuracy and rank == 0:
        if prec != _lib.PREC_FP64:
            h64 = _lib.Handle(csr, a, b, _lib.PREC_FP64)
            b64 = _lib.Block(h64, vecs, keep_a0=True)
            s64 = torch.cuda.ExternalStream(h64.stream())
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(s64)
            mom64 = b64.dos_moments(0, M)
            f1.record(s64)
            torch.cuda.synchronize()
            fp64_ms = f0.elapsed_time(f1)
            b64.close()
            h64.close()

            d32, d64 = dos_k(mom), dos_k(mom64)
            diff = np.abs(d32 - d64) / n
            # nodes inside the spectral bounds (the eps margin excluded):
            # there the DOS is nonzero; outside it the 1/sqrt(1 - x^2)
            # weight of the reconstruction amplifies rounding near zero DOS
            inside = np.abs(nodes) <= 1 - 0.05 / 2
            accuracy = {
                'dos_linf_per_orbital_vs_fp64': float(np.max(diff)),
                'dos_linf_per_orbital_vs_fp64_inside_bounds':
                    float(np.max(diff[inside])),
                'dos_linf_rel_vs_fp64': float(
                    np.max(np.abs(d32 - d64)) / np.max(np.abs(d64))),
                'argmax_node_x': float(nodes[int(np.argmax(diff))]),
                'reference': 'FP64 GPU path (parity-tested against the '
                             'reference fixtures at 1e-12)',
                'fp64_gpu_value': nnz * R * M / (fp64_ms / 1e3),
                'fp64_gpu_ms_per_step': fp64_ms,
                'mixed_over_fp64_moment_steps': fp64_ms / ms_per_step}

    # ---- CPU baseline (oracle port on the host cores) ----------------------
    cpu = None
    if args.cpu and rank == 0 and world == 1:
        procs = args.cpu_procs or os.cpu_count() or 1
        base = CpuBaseline(ham, a, b, vecs, procs)
        om = None
        try:
            base.run(8)  # spawn + load
            v, dt = base.run(args.ref_moments)
            k = min(args.oracle_vectors, R)
            if accuracy is not None and k > 0:
                # the oracle (complex128 scipy recursion of kwant.kpm's
                # algorithm) on the first k vectors at the full M, after the
                # timed CPU sample
                t0 = time.perf_counter()
                om = base.oracle_moments(vecs[:k], M)
                o_dt = time.perf_counter() - t0
        finally:
            base.close()
        if om is not None:
            from oracle import kpm_oracle as ko
            rho_o = ko.calc_fft_moments(ko.reduce_moments(om, a))[0]
            accuracy['oracle'] = {
                'vectors': int(k), 'moments': int(M),
                'dos_linf_per_orbital_vs_oracle': float(
                    np.max(np.abs(dos_k(mom[:k]) - rho_o)) / n),
                'fp64_gpu_dos_linf_per_orbital_vs_oracle': float(
                    np.max(np.abs(dos_k(mom64[:k]) - rho_o)) / n),
                'fp64_gpu_moments_rel_linf_vs_oracle': float(
                    np.max(np.abs(mom64[:k] - om)) / np.max(np.abs(om))),
                'oracle_s': o_dt,
                'reference': 'oracle port of kwant.kpm (complex128 scipy '
                             'recursion and its own reconstruction) on the '
                             'same Hamiltonian, vectors and (a, b), the '
                             'first %d vectors, all 2M nodes' % k}
        cpu = {'value': v, 'unit': UNIT, 'cores': procs, 'kind': 'port',
               'sample': '%d vectors x %d moments of the same workload, one '
                         'spawned process per vector (%.1f s; scipy\'s CSR '
                         'matvec is single-threaded)'
                         % (procs, args.ref_moments, dt),
               'cpu': _cpu_model()}

    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms_per_step, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None,
            'dtype': {'mixed': 'c64+bf16lo, f64acc', 'single': 'c64+f64acc',
                      'fp64': 'c128'}[args.precision],
            'data': 'synthetic',
            'config': {'workload': _workload_name(args),
                       'precision': args.precision, 'nnz': int(nnz),
                       'orbitals': int(n), 'R': R, 'M': M,
                       'matvec_steps_per_step': M // 2,
                       'l2': 'inputs larger than L2 (vector blocks %.2f GB '
                             'each), no flush' % (n * R * VEC_BYTES[
                                 args.precision] / 1e9),
                       'setup_s': setup_s, 'parallelism':
                       'replicas' if world > 1 else 'single'},
            'roofline': {'bound': 'hbm', 'achieved': achieved,
                         'peak': hbm_peak, 'unit': 'GB/s',
                         'frac': achieved / hbm_peak, 'traffic': traffic,
                         'kernel': {'mixed': 'cheb_step_hilo_kernel',
                                    'single': 'cheb_step_ell_kernel',
                                    'fp64': 'cheb_step_kernel'}[
                                        args.precision] +
                                   ' (fused step + moment dots)',
                         'algorithmic_bytes_per_launch': B,
                         'avg_launch_ms': avg_step_ms,
                         'launches_timed': n_step,
                         'peak_source': peak_src},
            'cpu_baseline': cpu, 'e2e': e2e, 'gpu_launches': launches,
            'clocks': clk, 'accuracy': accuracy,
        }
        if args.kubo and world == 1:
            # the Kubo-Bastin workload at its default size, so that every
            # default run measures it too (not part of this line's value)
            line['kubo'] = kubo_record(args, 5, 3, cpu=args.cpu,
                                       accuracy=args.accuracy)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    block.close()
    handle.close()
    return 0


def run_ldos(args):
    """Local DOS workload (not the headline line): the graphene system of
    the DOS workload with kwant.operator.Density on the 1000 sites nearest
    the flake's centre as the operator (one output per site), R vectors, M
    moments by the operator path (M - 1 matvecs, kwant/kpm.py:478-484).
    Metric as the DOS line: nnz * R * M / time of one moment run."""
    import torch
    from kwant_gb300 import _lib, kpm, lattices, operator
    syst = lattices.honeycomb(args.cells, t=1.0, flux=1.0 / 1000, W=0.5,
                              seed=0)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    n, nnz = ham.shape[0], ham.nnz
    centre = syst.positions.mean(axis=0)
    d = np.linalg.norm(syst.positions - centre, axis=1)
    where = np.sort(np.argsort(d)[:1000])
    dens = operator.Density(syst, where=list(where))
    R, M = args.vectors, args.moments
    _, v0, vecs = make_workload(args.cells, R)
    lo, hi = kpm.spectral_bounds(ham, 0.05, v0, 'lanczos')
    a, b = kpm._rescale_ab(lo, hi, 0.05)
    handle = _lib.Handle(_lib.Csr(ham), a, b, _lib.PREC_MIXED, reorder=True)
    op = _lib.Op(handle, operator.lower(dens))
    block = _lib.Block(handle, vecs, keep_a0=True)
    stream = torch.cuda.ExternalStream(handle.stream())

    def one_step():
        block.rewind()
        return block.op_moments(op, 0, M)

    for _ in range(args.warmup):
        one_step()
    handle.profile(True)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        mom = one_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    n_step, step_ms = handle.profile_read()
    handle.profile(False)
    ms = ev0.elapsed_time(ev1) / args.steps
    accuracy = None
    if args.accuracy:
        # FP64 GPU path on the first 8 vectors (parity-tested at 1e-12)
        k = min(8, R)
        h64 = _lib.Handle(_lib.Csr(ham), a, b, _lib.PREC_FP64)
        op64 = _lib.Op(h64, operator.lower(dens))
        b64 = _lib.Block(h64, vecs[:k], keep_a0=True)
        ref = b64.op_moments(op64, 0, M)
        nodes = kpm._chebyshev_nodes(2 * M)
        _, rho = _lib.reconstruct(mom[:k], True, True, a,
                                  _lib.KERNEL_JACKSON, 4.0, nodes)
        _, rho64 = _lib.reconstruct(ref, True, True, a,
                                    _lib.KERNEL_JACKSON, 4.0, nodes)
        inside = np.abs(nodes) <= (hi - lo) / (2 * a) * 0.999
        err = np.abs(rho.real - rho64.real)
        accuracy = {'ldos_linf_vs_fp64': float(err.max()),
                    'ldos_linf_vs_fp64_inside_bounds':
                    float(err[inside].max()),
                    'ldos_max': float(np.abs(rho64.real).max()),
                    'vectors_compared': k,
                    'reference': 'FP64 GPU path, same vectors and bounds, '
                                 'all 2M nodes (per site of the 1000)'}
        b64.close()
        op64.close()
        h64.close()
    peaks = {}
    pk = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get('hbm_gbs', 6800.0))
    # the operator path advances plain complex64 vectors (8 B per element)
    B = step_bytes(nnz, n, R, 'single')
    avg = step_ms / max(n_step, 1)
    achieved = B / (avg / 1e3) / 1e9
    line = {
        'metric': METRIC, 'value': nnz * R * M / (ms / 1e3), 'unit': UNIT,
        'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'c64+f64acc', 'data': 'synthetic',
        'config': {'workload': 'LDOS: honeycomb %dx%d cells, Density on the '
                               '1000 central sites, R=%d, M=%d'
                               % (args.cells, args.cells, R, M),
                   'nnz': int(nnz), 'orbitals': int(n), 'outputs': 1000},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': hbm,
                     'unit': 'GB/s', 'frac': achieved / hbm, 'traffic': None,
                     'kernel': 'cheb_step_ell_kernel (operator path, no '
                               'fused dots)',
                     'algorithmic_bytes_per_launch': B, 'avg_launch_ms': avg,
                     'launches_timed': n_step},
        'accuracy': accuracy,
    }
    if args.cpu:
        procs = args.cpu_procs or os.cpu_count() or 1
        base = CpuBaseline(ham, a, b, vecs, procs, where=list(where))
        try:
            base.run(4)  # spawn + load
            v, dt = base.run(args.ref_moments)
        finally:
            base.close()
        line['cpu_baseline'] = {
            'value': v, 'unit': UNIT, 'cores': procs, 'kind': 'port',
            'sample': '%d vectors x %d moments of the same workload (operator '
                      'path, Density on the 1000 sites), one spawned process '
                      'per vector (%.1f s)' % (procs, args.ref_moments, dt),
            'cpu': _cpu_model()}
    print(json.dumps(line))
    block.close()
    op.close()
    handle.close()
    return 0


# ------------------------------------------------------------ Kubo-Bastin
_KW = {}


def _kubo_cpu_init(path, lmin, lmax, M):
    import scipy.sparse as sp
    d = np.load(path)
    mk = lambda k: sp.csr_matrix((d[k + '_data'], d[k + '_indices'],
                                   d[k + '_indptr']), shape=tuple(d['shape']))
    _KW.update(ham=mk('h'), vx=mk('vx'), vy=mk('vy'), lmin=lmin, lmax=lmax,
               M=M)


def _kubo_cpu_task(vec):
    """The oracle port of kwant.kpm.conductivity's moments matrix
    (Correlator, kwant/kpm.py:557-606 and :685-695) for one vector."""
    from oracle import kpm_oracle as ko
    t0 = time.perf_counter()
    mu, _, _ = ko.correlator_moments_matrix(
        _KW['ham'], [vec], _KW['lmin'], _KW['lmax'], _KW['M'], _KW['vx'],
        _KW['vy'])
    return mu, time.perf_counter() - t0


def _sigma_grid(mu_mat, a, b, M, mus, temps):
    """sigma_xy(mu, T) over a grid from a moments matrix, with this
    package's device integral factor (kwant/kpm.py:720-760) and
    Fermi-weighted Simpson sums (kwant/kpm.py:608-630)."""
    from kwant_gb300 import _lib, kpm
    g = np.asarray(kpm.jackson_kernel(np.ones(M)), dtype=float)
    g[0] /= 2
    nodes = kpm._chebyshev_nodes(2 * M)
    factor = _lib.integral_factor(mu_mat, g, nodes)
    w = (2 * 4 ** 2 / (2 * a) ** 2) * kpm._simpson_weights(nodes) / \
        (1 - nodes ** 2) ** 2
    mm, tt = np.meshgrid(mus, temps, indexing='ij')
    out = _lib.fermi_sums(a * nodes + b, w, factor[:, None], mm.ravel(),
                          tt.ravel())
    return out.reshape(mm.shape)


def _rel_linf(x, ref):
    return float(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))


def kubo_record(args, steps, warmup, cpu=True, accuracy=True):
    """Kubo-Bastin workload: square L x L, two orbitals, t = 1, Rashba 0.3,
    exchange 0.2, W = 1 (seed 0), R vectors, M moments, sigma_xy.  A step is
    the device part of conductivity(): both Chebyshev recursions with
    stored vectors and the moments-matrix contraction on the tensor cores
    (BF16x3).  Accuracy: sigma_xy on a (mu, T) grid against the FP64 path
    (all R vectors) and against the oracle (the CPU sample's vectors); CPU
    baseline: the oracle's moments matrix, one spawned process per vector."""
    import torch
    from kwant_gb300 import _lib, kpm, lattices
    L, R, M = args.kubo_l, args.kubo_vectors, args.kubo_moments
    syst = lattices.rashba_square(L, t=1.0, alpha=0.3, exchange=0.2, W=1.0,
                                  seed=0)
    ham = syst.hamiltonian_submatrix(sparse=True).tocsr()
    n, nnz = ham.shape[0], ham.nnz
    pos = syst.orbital_positions()
    vx = kpm._velocity(ham, None, 'x', pos)
    vy = kpm._velocity(ham, None, 'y', pos)
    rng = np.random.RandomState(1)
    v0 = np.exp(2j * np.pi * rng.random_sample(n))
    vecs = np.exp(2j * np.pi * rng.random_sample((R, n)))
    lo, hi = kpm.spectral_bounds(ham, 0.05, v0, 'lanczos')
    a, b = kpm._rescale_ab(lo, hi, 0.05)
    _a = a * (1 - 0.05 / 2)
    a2, b2 = kpm._rescale_ab(b - _a, b + _a, 0.05)
    h = _lib.Handle(ham, a, b, _lib.PREC_MIXED, reorder=True)
    cva, cvb = _lib.Csr(vx), _lib.Csr(vy)
    stream = torch.cuda.ExternalStream(h.stream())

    def step(v=vecs, hd=h, gemm=1):
        return _lib.correlator_moments(hd, a2, b2, cva, cvb, v, M, gemm=gemm)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    launches0 = _lib.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    gem = []
    e0.record(stream)
    for _ in range(steps):
        mu = step()
        gem.append(h.last_gemm())
    e1.record(stream)
    torch.cuda.synchronize()
    launches = _lib.launch_count() - launches0
    ms = e0.elapsed_time(e1) / steps
    g_ms = float(np.median([g[0] for g in gem]))
    g_fl = gem[-1][1]
    peaks = {}
    pk = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    tpeak = float(peaks.get('bf16_tflops', 1900.0))
    achieved = g_fl / (g_ms / 1e3) / 1e12
    complex_flops = 8.0 * R * M * M * n
    rec = {
        'workload': 'kubo-bastin sigma_xy: rashba square %dx%d x2 orbitals, '
                    'R=%d, M=%d' % (L, L, R, M),
        'value': 2 * nnz * R * M / (ms / 1e3), 'unit': UNIT,
        'ms_per_step': ms, 'nnz': int(nnz), 'orbitals': int(n),
        'gpu_launches_per_step': launches / steps,
        'dtype': 'c64 recursion + bf16x3 GEMM',
        'roofline': {'bound': 'tensor', 'achieved': achieved, 'peak': tpeak,
                     'unit': 'TFLOP/s', 'frac': achieved / tpeak,
                     # ncu dram bytes of one launch on the 60 x 60 x 2,
                     # R = 16 case: 477.9 + 9.7 MB against 472.0 MB of
                     # operands (4 BF16 planes x M x K_pad x 2 operands),
                     # scaled
                     'traffic': (487.6 / 472.0) * 16.0 * M * g_fl /
                                (24.0 * M * M) if g_fl else None,
                     'kernel': 'bf16x3_tc_kernel',
                     'mma_flops_per_launch': g_fl, 'avg_launch_ms': g_ms,
                     'complex_equivalent_tflops':
                         complex_flops / (g_ms / 1e3) / 1e12,
                     'peak_source': 'measured' if 'bf16_tflops' in peaks
                     else 'fallback'},
    }
    mus = b + a * np.linspace(-0.8, 0.8, 17)
    temps = np.array([0.05, 0.2])
    if accuracy:
        h64 = _lib.Handle(ham, a, b, _lib.PREC_FP64)
        mu64 = step(hd=h64, gemm=0)
        s_mixed = _sigma_grid(mu, a, b, M, mus, temps)
        s_64 = _sigma_grid(mu64, a, b, M, mus, temps)
        rec['accuracy'] = {
            'mu_rel_linf_vs_fp64': _rel_linf(mu, mu64),
            'sigma_xy_rel_linf_vs_fp64': _rel_linf(s_mixed, s_64),
            'sigma_grid': '%d chemical potentials in b +- 0.8 a, T in %s'
                          % (len(mus), temps.tolist()),
            'reference': 'FP64 GPU path, all %d vectors' % R}
        # the same conductivity with FP16 hi/lo parts (gemm 'fp16x3': same
        # layout, MMAs and recursions), timed and checked alike
        step(gemm=4)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        mu16 = step(gemm=4)
        f1.record(stream)
        torch.cuda.synchronize()
        rec['accuracy']['fp16x3'] = {
            'ms_per_step': f0.elapsed_time(f1),
            'contraction_ms': h.last_gemm()[0],
            'mu_rel_linf_vs_fp64': _rel_linf(mu16, mu64),
            'sigma_xy_rel_linf_vs_fp64': _rel_linf(
                _sigma_grid(mu16, a, b, M, mus, temps), s_64)}
    if cpu:
        procs = min(args.cpu_procs or os.cpu_count() or 1, R)
        tmp = tempfile.NamedTemporaryFile(suffix='.npz', delete=False)
        tmp.close()
        np.savez(tmp.name, shape=np.array(ham.shape),
                 **{k + '_' + f: getattr(m, f) for k, m in
                    (('h', ham), ('vx', vx.tocsr()), ('vy', vy.tocsr()))
                    for f in ('data', 'indices', 'indptr')})
        pool = _spawn_pool(procs, _kubo_cpu_init, (tmp.name, lo, hi, M))
        try:
            pool.map(_kubo_cpu_task, [vecs[0]] * procs)   # spawn + load
            t0 = time.perf_counter()
            res = pool.map(_kubo_cpu_task, list(vecs[:procs]))
            dt = time.perf_counter() - t0
        finally:
            pool.close()
            pool.join()
            os.unlink(tmp.name)
        rec['cpu_baseline'] = {
            'value': 2 * nnz * procs * M / dt, 'unit': UNIT, 'cores': procs,
            'kind': 'port', 'sample': '%d vectors x %d moments of the same '
            'workload (both recursions and the moments matrix), one spawned '
            'process per vector (%.1f s)' % (procs, M, dt),
            'cpu': _cpu_model()}
        if accuracy:
            # sigma on the sample's vectors: oracle against both GPU paths
            from oracle import kpm_oracle as ko
            mu_o = np.mean([r[0] for r in res], axis=0)
            fac = ko.integral_factor(mu_o, a, b, M)
            s_o = np.array([[ko.conductivity_value(fac, a, b, M, m, t)
                             for t in temps] for m in mus])
            sub = vecs[:procs]
            mu_m = step(v=sub)
            mu_d = step(v=sub, hd=h64, gemm=0)
            rec['accuracy'].update({
                'sigma_xy_rel_linf_vs_oracle': _rel_linf(
                    _sigma_grid(mu_m, a, b, M, mus, temps), s_o),
                'sigma_xy_rel_linf_fp64_path_vs_oracle': _rel_linf(
                    _sigma_grid(mu_d, a, b, M, mus, temps), s_o),
                'mu_rel_linf_vs_oracle': _rel_linf(mu_m, mu_o),
                'oracle_vectors': procs})
    if accuracy:
        h64.close()
    h.close()
    return rec


def run_kubo(args):
    """The Kubo-Bastin workload as its own bench line (not the headline)."""
    rec = kubo_record(args, args.steps, args.warmup, cpu=args.cpu,
                      accuracy=args.accuracy)
    line = {
        'metric': METRIC, 'value': rec['value'], 'unit': UNIT, 'n_gpus': 1,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': rec['ms_per_step'], 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': rec['dtype'],
        'data': 'synthetic',
        'config': {'workload': rec['workload'], 'nnz': rec['nnz'],
                   'orbitals': rec['orbitals']},
        'roofline': rec['roofline'], 'cpu_baseline': rec.get('cpu_baseline'),
        'gpu_launches': int(rec['gpu_launches_per_step'] * args.steps),
        'accuracy': rec.get('accuracy'),
    }
    print(json.dumps(line))
    return 0


def run_batch(args):
    """Batched Wilson-Dirac workload (not the headline line): 32 disorder
    realisations (W ~ U[0, 3]) of L^3 cubic lattices with L ~ U{32..64}
    (seed 0), 4 orbitals, BSR 4 x 4, R = 256, M = 1024, complex64, all in
    one CUDA graph.  One step = one DOS run of every system."""
    from kwant_gb300 import batch
    rs = np.random.RandomState(args.batch_seed)
    S = args.batch_systems
    Ls = rs.randint(args.batch_lmin, args.batch_lmax + 1, size=S)
    Ws = rs.uniform(0.0, 3.0, size=S)
    R, M = args.batch_vectors, args.batch_moments
    bd = batch.BatchedDOS(R, M, seed=1)
    for s in range(S):
        bd.add_wilson_dirac(int(Ls[s]), m=1.5, W=float(Ws[s]), seed=100 + s)
    t0 = time.perf_counter()
    bd.moments()                       # prepare + autotune + capture + run
    prep_s = time.perf_counter() - t0
    times = []
    for _ in range(max(0, args.warmup - 1)):
        bd.moments()
    for _ in range(args.steps):
        bd.moments()
        times.append(bd.stats()[0])
    ms = float(np.median(times))
    _, nodes, vpl = bd.stats()
    fmt, ell_k = bd.step_format()
    order = bd.work_order()
    # Kwant CSR nnz (exact zeros dropped): 4 per site onsite, 8 per
    # directed hopping block (Gamma_0 diagonal + tau_x (x) sigma_j)
    nnz = int(sum(4 * L ** 3 + 8 * 6 * L * L * (L - 1) for L in Ls))
    orbs = int(sum(4 * L ** 3 for L in Ls))
    Rpad = -(-R // 32) * 32
    # algorithmic bytes per step: the stored matrix once (orbital-row ELL:
    # K entries of 4 + 8 bytes per row; BSR: 8 blocks of 4 + 128 bytes per
    # block row), 3 vector passes (x, alpha_{n-1}, out)
    if fmt == 1:
        mat = orbs * ell_k * 12
    elif fmt == 2:      # block columns + 16 entries (4 + 8 bytes) per row
        mat = int(sum(int(L) ** 3 * 8 * 4 for L in Ls)) + orbs * 16 * 12
    else:
        mat = int(sum(int(L) ** 3 * 8 * (4 + 16 * 8) for L in Ls))
    B = int(mat + 3 * orbs * Rpad * 8)
    steps = M // 2
    achieved = B * steps / (ms / 1e3) / 1e9
    peaks = {}
    pk = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get('hbm_gbs', 6800.0))
    line = {
        'metric': METRIC, 'value': nnz * R * M / (ms / 1e3), 'unit': UNIT,
        'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'c64+f64acc', 'data': 'synthetic',
        'config': {'workload': 'batched wilson-dirac: %d systems, L in '
                               '[%d, %d], W ~ U[0,3], R=%d, M=%d, one CUDA '
                               'graph' % (S, args.batch_lmin, args.batch_lmax,
                                          R, M),
                   'L': [int(x) for x in Ls], 'orbitals': orbs, 'nnz': nnz,
                   'graph_nodes': nodes, 'vectors_per_lane': vpl,
                   'work_order': order,
                   'step_format': ['BSR 4x4', 'orbital-row ELL, width %d'
                                   % ell_k,
                                   'sparse blocks (staged in shared memory)'
                                   ][fmt],
                   'prepare_s': prep_s},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': hbm,
                     'unit': 'GB/s', 'frac': achieved / hbm,
                     # ncu dram bytes of BSR launches on the 2-system
                     # (L = 37, 32) case against 2.138 GB algorithmic:
                     # 2.697 + 0.668 GB partition-major, 2.281 + 0.664 GB
                     # group-major; scaled by the algorithmic bytes
                     'traffic': B * ((2.697 + 0.668) / 2.138
                                     if order == 'partition' else
                                     (2.281 + 0.664) / 2.138)
                     if fmt == 0 else None,
                     'kernel': ['bsr_step_kernel', 'ell_batch_step_kernel',
                                'sb_step_kernel'][fmt] +
                               ' (+ finalize, per graph step)',
                     'algorithmic_bytes_per_step': B,
                     'avg_step_ms': ms / steps},
    }
    if args.accuracy:
        line['accuracy'] = batch_accuracy(bd, bd.moments(), Ls, Ws, R, M)
    if args.batch_mixed:
        # the compensated mode on the same systems and vectors (one warm-up
        # and one timed run: ~1 min each), after freeing the 'single' batch
        bd._b.close()
        del bd
        bm = batch.BatchedDOS(R, M, seed=1, precision='mixed')
        for s in range(S):
            bm.add_wilson_dirac(int(Ls[s]), m=1.5, W=float(Ws[s]),
                                seed=100 + s)
        bm.moments()
        mom = bm.moments()
        mms, launches, _ = bm.stats()
        Bm = int(mat_ell_mixed(Ls) + 3 * orbs * Rpad * 12)
        rec = {'precision': 'mixed (compensated single-system step, system '
                            'after system)',
               'value': nnz * R * M / (mms / 1e3), 'unit': UNIT,
               'ms_per_step': mms, 'gpu_launches_per_step': launches,
               'roofline': {'bound': 'hbm',
                            'achieved': Bm * steps / (mms / 1e3) / 1e9,
                            'peak': hbm, 'unit': 'GB/s',
                            'frac': Bm * steps / (mms / 1e3) / 1e9 / hbm,
                            'traffic': None,
                            'kernel': 'cheb_step_hilo_kernel (ELL width 16)',
                            'algorithmic_bytes_per_step': Bm}}
        if args.accuracy:
            rec['accuracy'] = batch_accuracy(bm, mom, Ls, Ws, R, M)
        bm.close()
        line['mixed'] = rec
    if args.cpu:
        line['cpu_baseline'] = batch_cpu(args, Ls, Ws, R, M,
                                         line.get('accuracy'))
    print(json.dumps(line))
    return 0


def batch_cpu(args, Ls, Ws, R, M, accuracy):
    """CPU baseline of the batched workload: the oracle port on the largest
    system of the batch (its Hamiltonian assembled on the host, exact zeros
    dropped as in Kwant's CSR), one spawned process per vector over 16
    vectors x 128 moments.  With accuracy, the oracle's FP64 moments of the
    smallest system's first 16 device-generated vectors at the full M pin
    the FP64 GPU path that the batch's own accuracy figures are measured
    against."""
    from kwant_gb300 import _lib, batch
    procs = args.cpu_procs or os.cpu_count() or 1
    big = int(np.argmax(Ls))
    H = batch.wilson_dirac_matrix(int(Ls[big]), 1.5, float(Ws[big]), 100 + big)
    H.eliminate_zeros()
    n = H.shape[0]
    g = float(np.max(np.asarray(abs(H).sum(axis=1))))
    a, b = g / (1 - 0.05 / 2), 0.0
    vecs = batch.random_phase_vectors(1, big, procs, n).astype(complex)
    base = CpuBaseline(H, a, b, vecs, procs)
    try:
        base.run(8)  # spawn + load
        v, dt = base.run(args.batch_cpu_moments)
    finally:
        base.close()
    out = {'value': v, 'unit': UNIT, 'cores': procs, 'kind': 'port',
           'sample': '%d vectors x %d moments of the largest system (L = '
                     '%d, %d orbitals), one spawned process per vector '
                     '(%.1f s)' % (procs, args.batch_cpu_moments,
                                   int(Ls[big]), n, dt),
           'cpu': _cpu_model()}
    if accuracy is not None and args.oracle_vectors > 0:
        s = int(np.argmin(Ls))
        Hs = batch.wilson_dirac_matrix(int(Ls[s]), 1.5, float(Ws[s]), 100 + s)
        Hs.eliminate_zeros()
        k = min(args.oracle_vectors, R, procs)
        vs = batch.random_phase_vectors(1, s, k, Hs.shape[0]).astype(complex)
        gs = float(np.max(np.asarray(abs(Hs).sum(axis=1))))
        a_s, b_s = gs / (1 - 0.05 / 2), 0.0
        ob = CpuBaseline(Hs, a_s, b_s, vs, k)
        try:
            om = ob.oracle_moments(vs, M)
        finally:
            ob.close()
        m64 = _lib.dos(Hs, a_s, b_s, _lib.PREC_FP64, vs, M)[0]
        accuracy['oracle'] = {
            'system': 'smallest (L = %d)' % int(Ls[s]), 'vectors': int(k),
            'moments': int(M),
            'fp64_gpu_moments_rel_linf_vs_oracle': float(
                np.max(np.abs(m64 - om)) / np.max(np.abs(om))),
            'reference': 'oracle port of kwant.kpm (complex128 scipy '
                         'recursion) on the same Hamiltonian and vectors'}
    return out


def mat_ell_mixed(Ls):
    """Matrix bytes of one compensated ELL step over the batch: 16
    entries per orbital row (13 non-zeros padded), 4 + 8 bytes each."""
    return int(sum(4 * int(L) ** 3 for L in Ls)) * 16 * 12


def batch_accuracy(bd, mom, Ls, Ws, R, M):
    """Per-orbital DOS of the smallest system of the batch against the
    FP64 GPU path (parity-tested against the reference fixtures) on the
    same Hamiltonian (the device generator's disorder assembled on the
    host), the same device-generated vectors and the same bounds, at all
    2M Chebyshev nodes (untimed)."""
    from kwant_gb300 import _lib, batch
    from kwant_gb300.kpm import _chebyshev_nodes as kpm_nodes
    s = int(np.argmin(Ls))
    L, W = int(Ls[s]), float(Ws[s])
    H = batch.wilson_dirac_matrix(L, 1.5, W, 100 + s)
    n = H.shape[0]
    a, b = bd.scales[s]
    vecs = batch.random_phase_vectors(1, s, R, n)
    mom64 = _lib.dos(H, a, b, _lib.PREC_FP64, vecs, M)[0].mean(axis=0)
    ref = mom.copy()
    ref[s] = mom64
    _, rho = bd.densities(mom)
    _, rho64 = bd.densities(ref)
    err = np.abs(rho[s] - rho64[s]) / n
    return {'dos_linf_per_orbital_vs_fp64': float(err.max()),
            'argmax_node_x': float(kpm_nodes(2 * M)[np.argmax(err)]),
            'system': {'L': L, 'W': W, 'orbitals': int(n)},
            'reference': 'FP64 GPU path, same vectors and bounds, all 2M '
                         'nodes'}


def run_surrogate(args):
    """Learned-moment-surrogate workload (not the headline line): the
    honeycomb family over W in [0, 3], flux in [0, 0.02], mass in [0, 0.3]
    on 500 x 500 cells; 4096 training points (3584 fit + 512 calibration)
    and 1024 held-out points, M = 512, R = 32 (complex64 recursion).  The
    held-out sweep runs twice: plain KPM at every point, and surrogate with
    KPM fallback where the estimated DOS error exceeds the tolerance."""
    from kwant_gb300 import lattices, surrogate as S
    box = ((0.0, 0.02), (0.0, 3.0), (0.0, 0.3))
    M, R = args.sur_moments, args.sur_vectors
    t0 = time.perf_counter()
    fam = lattices.honeycomb_family(args.sur_cells, seed=0)
    # plain complex64 recursion: the DOS is compared at |x| <= 0.95, where it
    # is within ~3e-7 of the FP64 path, far below the R = 32 stochastic
    # error (~6e-4) that bounds every tolerance here; the compensated step
    # would cost 1.6x the time per point for no visible difference
    sweep = S.MomentSweep(fam, box, num_moments=M, num_vectors=R,
                          precision='single', rng=1)
    A, _ = S.dos_operator(M, sweep.a, sweep.b)
    setup_s = time.perf_counter() - t0
    Xtr = S.random_points(box, args.sur_train, 11)
    Xte = S.random_points(box, args.sur_test, 12)
    sweep.moments(Xtr[:max(3, args.warmup)])            # warm-up
    t0 = time.perf_counter()
    Ytr = sweep.moments(Xtr)
    gen_s = time.perf_counter() - t0
    ncal = min(512, args.sur_train // 8)
    sur = S.MomentSurrogate(box, M, members=args.sur_members, seed=1,
                            input_map=('sqrt', 'linear', 'linear'))
    t0 = time.perf_counter()
    losses = sur.fit(Xtr[:-ncal], Ytr[:-ncal], epochs=args.sur_epochs,
                     batch=256, lr=1e-3)
    train_s = time.perf_counter() - t0
    cal_err, cal_spread = sur.calibrate(Xtr[-ncal:], Ytr[-ncal:], A)
    # plain sweep of the held-out points (also the reference of the errors)
    t0 = time.perf_counter()
    Yte = sweep.moments(Xte)
    plain_s = time.perf_counter() - t0
    hybrid = S.SurrogateSweep(sur, sweep, A, tol=args.sur_tol)
    t0 = time.perf_counter()
    mom, accept, info = hybrid.run(Xte)
    hybrid_s = time.perf_counter() - t0
    err = np.abs((mom - Yte) @ A.T).max(axis=1)
    sur_only = sur.predict(Xte, A)[0]
    err_sur = np.abs((sur_only - Yte) @ A.T).max(axis=1)
    est = info['estimate']
    per_pt = plain_s / len(Xte)
    curve = []
    for tol in (1e-4, 3e-4, 1e-3, 3e-3, 1e-2, 3e-2):
        acc = est <= tol
        curve.append({'tol': tol, 'accepted': float(acc.mean()),
                      'max_err_accepted': float(err_sur[acc].max())
                      if acc.any() else None,
                      'frac_accepted_within_tol': float(
                          (err_sur[acc] <= tol).mean()) if acc.any() else None,
                      'sweep_s_model': info['surrogate_s'] +
                      float((~acc).sum()) * per_pt})
    # stochastic error of the plain sweep itself (spread over its vectors)
    pv = sweep.moments(Xte[:16], per_vector=True).real
    noise = (np.std(pv @ A.T, axis=1, ddof=1) / np.sqrt(R)).max(axis=1)
    n = len(Xte)
    # the smallest tolerance at which surrogate + KPM check beats the plain
    # sweep with >= 95 % of the accepted points really within it
    wins = [c['tol'] for c in curve if c['sweep_s_model'] < plain_s and
            c['accepted'] > 0 and c['frac_accepted_within_tol'] >= 0.95]
    verdict = {
        'configured_tol': args.sur_tol,
        'hybrid_beats_plain_at_configured_tol': hybrid_s < plain_s,
        'first_winning_tol': min(wins) if wins else None,
        'kpm_noise_linf_median': float(np.median(noise)),
        'configured_tol_below_kpm_noise':
            args.sur_tol < float(np.median(noise)),
        'note': 'the plain sweep (R vectors) is itself uncertain by its '
                'stochastic DOS error; a tolerance below it cannot be '
                'certified by the R-vector KPM check of the surrogate'}
    line = {
        'metric': 'held-out sweep points/s at DOS Linf error <= tol '
                  '(surrogate + KPM fallback)',
        'value': n / hybrid_s, 'unit': 'points/s', 'n_gpus': 1,
        'steps': 1, 'warmup': max(3, args.warmup),
        'ms_per_step': hybrid_s * 1e3, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'bf16 mlp + c64/f64acc kpm', 'data': 'synthetic',
        'config': {'workload': 'surrogate sweep: honeycomb %dx%d, W in '
                               '[0,3], flux in [0,0.02], mass in [0,0.3], '
                               'M=%d, R=%d' % (args.sur_cells,
                                               args.sur_cells, M, R),
                   'train_points': args.sur_train, 'fit_points':
                   args.sur_train - ncal, 'calibration_points': ncal,
                   'heldout_points': n, 'members': args.sur_members,
                   'epochs': args.sur_epochs, 'tol': args.sur_tol,
                   'dos_units': 'per site per unit energy, Jackson, '
                                '|x| <= 0.95'},
        'plain_sweep': {'points_per_s': n / plain_s, 'seconds': plain_s,
                        'ms_per_point': per_pt * 1e3},
        'hybrid_sweep': {'seconds': hybrid_s, 'accepted':
                         float(accept.mean()), 'kpm_points':
                         int((~accept).sum()), 'max_err':
                         float(err.max()), 'surrogate_s':
                         info['surrogate_s'], 'kpm_s': info['kpm_s']},
        'surrogate_only': {'err_median': float(np.median(err_sur)),
                           'err_p10': float(np.quantile(err_sur, 0.1)),
                           'err_p90': float(np.quantile(err_sur, 0.9)),
                           'err_max': float(err_sur.max()),
                           'estimate_scale': sur.scale,
                           'estimate_median': float(np.median(est))},
        'tolerance_curve': curve,
        'tolerance_verdict': verdict,
        'kpm_noise_linf_median': float(np.median(noise)),
        'costs_s': {'setup': setup_s, 'dataset': gen_s, 'train': train_s,
                    'train_loss': [float(x) for x in losses]},
    }
    if args.cpu:
        # the reference has no surrogate: its sweep is the plain KPM at every
        # point; the oracle port on the first held-out point's Hamiltonian
        # (host assembly of the family), one spawned process per vector
        procs = min(args.cpu_procs or os.cpu_count() or 1, R)
        H = fam.hamiltonian(*Xte[0])
        vecs = np.exp(2j * np.pi * np.random.RandomState(3)
                      .random_sample((procs, H.shape[0])))
        base = CpuBaseline(H, sweep.a, sweep.b, vecs, procs)
        try:
            base.run(8)  # spawn + load
            _, dt = base.run(M)
        finally:
            base.close()
        pt_s = dt * R / procs
        line['cpu_baseline'] = {
            'value': 1.0 / pt_s, 'unit': 'points/s', 'cores': procs,
            'kind': 'port',
            'sample': '%d of the %d vectors x %d moments of one held-out '
                      'point (%.1f s), scaled to the point\'s %d vectors; '
                      'plain KPM at every point (no surrogate)'
                      % (procs, R, M, dt, R),
            'cpu': _cpu_model()}
    print(json.dumps(line))
    return 0


def main():
    p = argparse.ArgumentParser()
    p.add_argument('--workload', default='dos', choices=['dos', 'kubo',
                                                         'batch',
                                                         'surrogate',
                                                         'ldos'])
    p.add_argument('--sur-cells', type=int, default=500)
    p.add_argument('--sur-moments', type=int, default=512)
    p.add_argument('--sur-vectors', type=int, default=32)
    p.add_argument('--sur-train', type=int, default=4096)
    p.add_argument('--sur-test', type=int, default=1024)
    p.add_argument('--sur-members', type=int, default=4)
    p.add_argument('--sur-epochs', type=int, default=2000)
    p.add_argument('--sur-tol', type=float, default=1e-4)
    p.add_argument('--batch-systems', type=int, default=32)
    p.add_argument('--batch-lmin', type=int, default=32)
    p.add_argument('--batch-lmax', type=int, default=64)
    p.add_argument('--batch-vectors', type=int, default=256)
    p.add_argument('--batch-moments', type=int, default=1024)
    p.add_argument('--batch-seed', type=int, default=0)
    p.add_argument('--no-batch-mixed', dest='batch_mixed',
                   action='store_false',
                   help='leave the compensated batch sub-record out')
    p.add_argument('--kubo-l', type=int, default=200)
    p.add_argument('--kubo-vectors', type=int, default=16)
    p.add_argument('--kubo-moments', type=int, default=256)
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=5)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    p.add_argument('--precision', default='mixed',
                   choices=['mixed', 'single', 'fp64'])
    p.add_argument('--cells', type=int, default=1000)
    p.add_argument('--vectors', type=int, default=64)
    p.add_argument('--moments', type=int, default=2000)
    p.add_argument('--ref-moments', type=int, default=100)
    p.add_argument('--batch-cpu-moments', type=int, default=128)
    p.add_argument('--oracle-vectors', type=int, default=16,
                   help='vectors of the headline DOS run checked against '
                        'the oracle at the full M (0: none)')
    p.add_argument('--cpu-procs', type=int, default=0)
    p.add_argument('--no-e2e', dest='e2e', action='store_false')
    p.add_argument('--no-cpu', dest='cpu', action='store_false')
    p.add_argument('--no-accuracy', dest='accuracy', action='store_false')
    p.add_argument('--no-reorder', dest='reorder', action='store_false')
    p.add_argument('--no-kubo', dest='kubo', action='store_false',
                   help='leave the Kubo-Bastin sub-record out of the DOS line')
    args = p.parse_args()
    if args.warmup < 3 and args.impl == 'ours':
        print('warning: fewer than 3 warm-up steps', file=sys.stderr)
    if args.impl == 'reference':
        return run_reference(args)
    if args.workload == 'kubo':
        return run_kubo(args)
    if args.workload == 'batch':
        return run_batch(args)
    if args.workload == 'surrogate':
        return run_surrogate(args)
    if args.workload == 'ldos':
        return run_ldos(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
