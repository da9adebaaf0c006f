"""`bench.py --impl reference` runs on the host cores only: its JSON line
(the contract the reference arm must keep) is checked here without a GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_line(workload):
  env = dict(os.environ, GBM_REFERENCE_SECONDS='1')
  out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference',
                        '--workload', workload, '--steps', '1', '--warmup', '0'],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
  assert out.returncode == 0, out.stderr[-2000:]
  lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
  assert len(lines) == 1, out.stdout
  return json.loads(lines[0])


@pytest.mark.parametrize('workload', ['hmc_logreg_1000x25', 'nuts_logreg_1e5x100'])
def test_reference_line_contract(workload):
  d = _reference_line(workload)
  assert d['impl'] == 'reference'
  assert d['unit'] == 'grad-evals/s' and d['higher_is_better'] is True
  assert d['value'] > 0 and d['steps'] >= 1
  assert d['config']['workload'] == workload
  cb = d['cpu_baseline']
  assert cb['kind'] == 'port' and cb['cores'] >= 1 and cb['value'] == d['value'] and cb['sample']
  assert d['e2e'] == {'value': d['value'], 'unit': 'grad-evals/s', 'h2d_bytes_per_step': 0,
                      'd2h_bytes_per_step': 0}


def test_reference_serving_is_unavailable():
  d = _reference_line('serve_logreg_stream')
  assert d['impl'] == 'reference' and d['unavailable']
