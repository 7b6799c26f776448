"""The benchmark line's contract, checked on the CPU through the reference
arm (the oracle program timed on the host): one JSON line with the keys the
GPU arm prints, impl "reference", an e2e with no host-device copies, a
cpu_baseline describing the run, and the same config dict as the GPU arm for
the same workload."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better', 'scaling',
        'vs_baseline', 'dtype', 'data', 'config', 'cpu_baseline', 'e2e')


@pytest.mark.skipif(subprocess.run(['which', 'g++'], capture_output=True).returncode != 0, reason='needs g++')
def test_reference_arm_line():
    r = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--size', '40', '--steps', '2',
                        '--warmup', '3', '--cpu-single-build'], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.strip().splitlines() if l.startswith('{')]
    assert len(lines) == 1, r.stdout[-2000:]
    line = json.loads(lines[0])
    for k in KEYS:
        assert k in line, k
    assert line['impl'] == 'reference' and line['value'] > 0 and line['higher_is_better'] is True
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['e2e']['d2h_bytes_per_step'] == 0
    assert line['e2e']['value'] == line['value'] and line['cpu_baseline']['value'] == line['value']
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] >= 1 and cb['sample']
    sys.path.insert(0, ROOT)
    import bench
    assert line['config'] == bench.elastic_config(40, 4, 'f32', 1, 0)
