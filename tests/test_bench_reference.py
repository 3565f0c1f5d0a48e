"""bench.py's reference arm (the oracle port of kwant.kpm on the host cores)
runs without a GPU and prints the contract's JSON line; ranks other than 0
exit quietly.  A small honeycomb flake keeps it to seconds."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, 'bench.py', '--impl', 'reference', '--cells', '30',
        '--steps', '1', '--warmup', '1', '--cpu-procs', '2',
        '--ref-moments', '20']


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    out = subprocess.run(ARGS, cwd=ROOT, env=env, capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    return out.stdout


def test_reference_arm_line():
    lines = [l for l in _run({}).splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['impl'] == 'reference'
    assert d['metric'] == 'KPM nnz*vec*moment/s' and d['value'] > 0
    assert d['higher_is_better'] is True and d['steps'] == 1
    assert d['cpu_baseline']['kind'] == 'port'
    assert d['cpu_baseline']['cores'] == 2
    assert d['cpu_baseline']['value'] == d['value']
    assert d['e2e']['h2d_bytes_per_step'] == 0
    assert d['e2e']['d2h_bytes_per_step'] == 0
    assert d['config']['M'] == 20


def test_reference_arm_other_ranks_exit_quietly():
    out = _run({'RANK': '1', 'WORLD_SIZE': '2'})
    assert not [l for l in out.splitlines() if l.startswith('{')]
