"""Build the kwant_gb300 CUDA library (sm_103a) in-tree.

Compiles every ``csrc/*.cu`` translation unit with nvcc in parallel and links
``kwant_gb300/libkwant_gb300.so`` (CUDA runtime linked statically, so the
library only needs the driver at run time).  Object files go to
``kwant_gb300/_build/``.  Rebuilds only what changed.

``build(variant='check')`` builds the bounds-checked debug library
(``-DKPM_CHECK``: the step kernels validate every gathered column index)
into ``kwant_gb300/_build_check/libkwant_gb300.so``; the package loads it
when the environment variable ``KWANT_GB300_LIB`` names it.
"""

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libkwant_gb300.so')
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
              '-Xcompiler', '-fvisibility=hidden', '--expt-relaxed-constexpr',
              '-I' + INCLUDE]


def _nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'),
                 '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _deps_mtime():
    files = glob.glob(os.path.join(CSRC, '*.cuh')) + \
        glob.glob(os.path.join(INCLUDE, '*.h'))
    return max(os.path.getmtime(f) for f in files) if files else 0


def _compile(nvcc, src, obj, extra):
    cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ['-c', src, '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s'
                           % (os.path.basename(src), r.stdout, r.stderr))
    return r.stderr


def build(verbose=False, extra_flags=(), variant=None):
    if variant == 'check':
        return _build(os.path.join(HERE, '_build_check'),
                      os.path.join(HERE, '_build_check', 'libkwant_gb300.so'),
                      verbose, list(extra_flags) + ['-DKPM_CHECK'])
    if variant is not None:
        raise ValueError('unknown build variant %r' % (variant,))
    return _build(BUILD, LIB, verbose, extra_flags)


def _build(BUILD, LIB, verbose, extra_flags):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    dep_t = _deps_mtime()
    # objects built with other flags are stale too
    stamp = os.path.join(BUILD, 'flags.txt')
    flags = ' '.join(ARCH + NVCC_FLAGS + list(extra_flags))
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        for o in glob.glob(os.path.join(BUILD, '*.o')):
            os.remove(o)
        with open(stamp, 'w') as f:
            f.write(flags)
    jobs = []
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
        objs.append(obj)
        if (not os.path.exists(obj) or os.path.getmtime(obj) <
                max(os.path.getmtime(src), dep_t)):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs),
                                                   os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, list(extra_flags))
                    for s, o in jobs]
            for f in futs:
                msg = f.result()
                if verbose and msg:
                    print(msg, file=sys.stderr)
    if jobs or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc] + ARCH + ['-shared', '-o', LIB] + objs + \
            ['-cudart', 'static']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed:\n%s\n%s' % (r.stdout, r.stderr))
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
