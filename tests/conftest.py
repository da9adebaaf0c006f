import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)


def pytest_configure(config):
  config.addinivalue_line(
      'markers', 'gpu: needs a CUDA GPU (sm_103a) and the built extension')


def pytest_collection_modifyitems(config, items):
  # Run GPU parity tests in file order; nothing else to reorder.
  return


@pytest.fixture(scope='session')
def golden_dir():
  return os.path.join(ROOT, 'tests', 'golden')
