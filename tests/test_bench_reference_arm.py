"""bench.py's reference arm on the host cores (the CPU port of the reference algorithm): one bounded step (a sample of
one batched state) prints the contract's JSON line (impl, metric, value, unit, cpu_baseline with kind/cores/sample,
e2e without copies) and loads no native library of this repository."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_its_line():
    r = subprocess.run([sys.executable, str(ROOT / 'bench.py'), '--impl', 'reference', '--steps', '1', '--warmup',
                        '0'], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith('{')][-1])
    assert line['impl'] == 'reference' and line['unit'] == 'solves/s' and line['higher_is_better'] is True
    assert line['value'] > 0 and line['steps'] == 1 and line['n_gpus'] == 1
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] >= 1 and cb['value'] == line['value'] and cb['sample']
    assert line['e2e'] == dict(value=line['value'], unit='solves/s', h2d_bytes_per_step=0, d2h_bytes_per_step=0)
    assert cb['native_libraries_loaded'] == []  # the CPU arm builds its geometry with the NumPy restatements
    assert cb['nproc'] >= cb['cores'] >= 1
