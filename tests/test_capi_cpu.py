"""C-ABI library checks that need no GPU: it loads, exports every symbol
include/gb300_mcmc.h declares, and the host-side pieces agree with the
reference's golden vectors."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
  syms = set()
  inc = os.path.join(ROOT, 'include')
  for f in os.listdir(inc):
    if f.endswith('.h'):
      src = open(os.path.join(inc, f)).read()
      src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
      syms |= set(re.findall(r'^\s*(?:GBM_API\s+)?(?:const\s+)?\w+\**\s+\**(gbm_\w+)\s*\(', src, re.M))
  return syms


@pytest.fixture(scope='module')
def libpath():
  from probability_gb300 import _native
  if not os.path.exists(_native.library_path()):
    from probability_gb300 import build
    build.build()
  return _native.library_path()


def test_library_exports_every_declared_symbol(libpath):
  lib = ctypes.CDLL(libpath)
  declared = _declared_symbols()
  assert len(declared) >= 15
  for name in declared:
    assert hasattr(lib, name), name
  from probability_gb300 import _native
  assert set(_native.exported_symbols()) <= declared


def test_host_only_entry_points(libpath):
  from probability_gb300 import _native
  lib = _native.lib()
  assert lib.gbm_version() >= 100
  out = (ctypes.c_uint32 * 2)()
  assert lib.gbm_step_key(_native.seed_words((7, 9)), 3, out) == 0
  from oracle import philox
  assert (out[0], out[1]) == philox.step_key((7, 9), 3)
  # Argument errors are reported, not crashed on.
  assert lib.gbm_nuts_create(None, 1, 10, 1000.0, 1, None) == _native.GBM_EINVAL
  assert b'NULL' in lib.gbm_last_error()
  # The free-running entry points validate before touching a device.
  assert lib.gbm_nuts_set_free_running(None, 1) == _native.GBM_EINVAL
  assert b'NULL' in lib.gbm_last_error()
  i64 = ctypes.c_int64()
  assert lib.gbm_nuts_run_free(None, 8, None, None, None, None, 0, _native.seed_words((1, 2)),
                               0, 4, 100, None, None, None, None, None, None, None,
                               ctypes.byref(i64)) == _native.GBM_EINVAL
  assert b'NULL' in lib.gbm_last_error()


def test_python_instruction_tables_match_reference(golden_dir):
  from probability_gb300.mcmc import nuts
  tables = json.load(open(os.path.join(golden_dir, 'nuts_instructions.json')))
  for depth in ('1', '4', '7', '10'):
    instr = nuts.build_tree_uturn_instruction(int(depth), init_memory=-1)
    w, r = nuts.generate_efficient_write_read_instruction(instr)
    assert w.tolist() == tables[depth]['write']
    assert r.tolist() == tables[depth]['read']


def test_kernel_rejects_unknown_target():
  from probability_gb300 import mcmc
  with pytest.raises(NotImplementedError):
    mcmc.NoUTurnSampler(lambda x: x, step_size=0.1)
  with pytest.raises(ValueError):
    mcmc.NoUTurnSampler(lambda x: x, step_size=0.1, max_tree_depth=0)


def test_seed_sanitizing():
  from probability_gb300 import _util
  assert _util.sanitize_seed(5) == (5, 0)
  assert _util.sanitize_seed((1, 2)) == (1, 2)
  assert _util.sanitize_seed(np.array([3, 4])) == (3, 4)
  with pytest.raises(ValueError):
    _util.sanitize_seed([1, 2, 3])
