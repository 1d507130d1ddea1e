"""The bench's reference arm on the CPU: one JSON line with the keys of the
measurement contract, and silence on ranks other than 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env):
    env = dict(os.environ, **extra_env)
    env['PYTHONPATH'] = ROOT + os.pathsep + env.get('PYTHONPATH', '')
    return subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                           '--warmup', '3', '--ref-seconds', '0.2', '--nodes', '101'],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=240)


def test_reference_arm_prints_one_contract_line():
    out = _run({})
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    d = json.loads(lines[-1])
    assert d['impl'] == 'reference'
    for k in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'higher_is_better', 'scaling',
              'vs_baseline', 'dtype', 'data', 'config', 'cpu_baseline', 'e2e'):
        assert k in d, k
    assert d['value'] > 0 and d['unit'] == 'elem/s' and d['higher_is_better'] is True
    assert d['steps'] == 1 and d['warmup'] == 3 and d['n_gpus'] == 1
    assert d['config']['workload'] == 'quad4_kc0_plate_101x101_nodes'
    cb = d['cpu_baseline']
    assert cb['kind'] in ('port', 'reference') and cb['cores'] >= 1 and cb['sample']
    assert cb['value'] == d['value']
    e2e = d['e2e']
    assert e2e['value'] == d['value'] and e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0


def test_reference_arm_other_ranks_exit_without_output():
    out = _run({'RANK': '1', 'WORLD_SIZE': '2', 'LOCAL_RANK': '1'})
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ''
