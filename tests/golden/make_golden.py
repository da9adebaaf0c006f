"""Regenerate the golden fixtures in this directory from the reference.

Run from the repository root, naming the root of a reference checkout
(the directory that holds ``tensorflow_probability/``):

    python tests/golden/make_golden.py <reference-root>

TensorFlow is not installed here, so the reference's ``nuts.py`` cannot be
imported as a module.  Its two instruction-table builders
(``build_tree_uturn_instruction``, ``generate_efficient_write_read_instruction``,
tensorflow_probability/python/mcmc/nuts.py:1013-1071) are plain NumPy, so this
script extracts exactly those two function definitions with ``ast`` and runs
them to produce the write/read tables for every depth 1..12.  The
dual-averaging constants are read from the reference's own test file
(dual_averaging_step_size_adaptation_test.py:47-57).  The Philox4x32-10
known-answer vectors are the published Random123 ones.
"""
import ast
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _extract_functions(path, names):
  src = open(path).read()
  tree = ast.parse(src)
  keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
  mod = ast.Module(body=keep, type_ignores=[])
  ns = {'np': np}
  exec(compile(mod, path, 'exec'), ns)
  return ns


def main(ref_root):
  mcmc = os.path.join(ref_root, 'tensorflow_probability', 'python', 'mcmc')
  ns = _extract_functions(os.path.join(mcmc, 'nuts.py'),
                          {'build_tree_uturn_instruction',
                           'generate_efficient_write_read_instruction'})
  tables = {}
  for depth in range(1, 13):
    instr = ns['build_tree_uturn_instruction'](depth, init_memory=-1)
    w, r = ns['generate_efficient_write_read_instruction'](instr)
    tables[str(depth)] = dict(write=[int(v) for v in w],
                              read=[[int(a), int(b)] for a, b in r])
  with open(os.path.join(HERE, 'nuts_instructions.json'), 'w') as f:
    json.dump(tables, f, separators=(',', ':'))

  test_src = open(os.path.join(
      mcmc, 'dual_averaging_step_size_adaptation_test.py')).read()
  consts = {m.group(1): float(m.group(2)) for m in
            re.finditer(r'^(_UPDATE_\w+) = ([0-9.]+)', test_src, re.M)}
  comments = {m.group(1): float(m.group(2)) for m in
              re.finditer(r'^(_UPDATE_\w+) = [0-9.]+\s+# err = ([-+0-9.]+)',
                          test_src, re.M)}
  da = dict(initial_t=10.0, exploration_shrinkage=0.05, target=0.75,
            cases=[dict(name=k, err=comments[k], expected=v)
                   for k, v in consts.items()])
  with open(os.path.join(HERE, 'dual_averaging.json'), 'w') as f:
    json.dump(da, f, indent=1)

  kat = [
      dict(key=[0, 0], ctr=[0, 0, 0, 0],
           out=[0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
      dict(key=[0xffffffff, 0xffffffff], ctr=[0xffffffff] * 4,
           out=[0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
      dict(key=[0xa4093822, 0x299f31d0],
           ctr=[0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
           out=[0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
  ]
  with open(os.path.join(HERE, 'philox_kat.json'), 'w') as f:
    json.dump(kat, f, indent=1)


if __name__ == '__main__':
  if len(sys.argv) != 2:
    sys.exit('usage: python tests/golden/make_golden.py <reference-root>')
  main(sys.argv[1])
