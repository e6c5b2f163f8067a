"""The benchmark's reference arm on the host cores (no GPU): `bench.py --impl reference`
prints the one JSON line the benchmark contract asks for, on the same metric and workload
as the CUDA arm, and under torchrun only rank 0 works."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def run_bench(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), *args], cwd=ROOT, env=e,
                          capture_output=True, text=True, timeout=900)


def test_reference_arm_prints_the_contract_line():
    p = run_bench(['--impl', 'reference', '--steps', '1', '--warmup', '1'])
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith('{')]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d['impl'] == 'reference'
    assert d['metric'] == bench.METRIC and d['unit'] == 'photons/s' and d['higher_is_better'] is True
    assert d['n_gpus'] == 1 and d['steps'] == 1 and d['warmup'] == 1
    assert d['value'] > 0 and d['ms_per_step'] > 0
    # the whole workload of the CUDA arm each step
    assert d['config']['photons_per_gpu'] == bench.N_PER_GPU
    assert d['config']['photons_per_step'] == bench.N_PER_GPU
    e2e = d['e2e']
    assert e2e['value'] == d['value'] and e2e['unit'] == d['unit']
    assert e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0
    cb = d['cpu_baseline']
    assert cb['kind'] in ('port', 'reference') and cb['cores'] >= 1 and cb['value'] == d['value']
    assert cb['sample']


def test_reference_arm_other_ranks_exit_without_work():
    p = run_bench(['--impl', 'reference', '--gpus', '2', '--steps', '1', '--warmup', '1'],
                  env={'RANK': '1', 'WORLD_SIZE': '2', 'LOCAL_RANK': '1'})
    assert p.returncode == 0, p.stderr[-2000:]
    assert not p.stdout.strip()
