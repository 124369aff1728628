import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)

# Location of the reference checkout (brax 0.14.2): $BRAXG_REFERENCE, else a
# checkout named `reference` beside this repository.  Only CPU-side golden
# tests read its fixture models, and they skip when it is absent.
REF = os.environ.get('BRAXG_REFERENCE') or os.path.join(os.path.dirname(ROOT), 'reference')


def pytest_configure(config):
  config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300)')


@pytest.fixture(scope='session')
def ref_path():
  if not os.path.isdir(os.path.join(REF, 'brax')):
    pytest.skip('reference checkout not present')
  return REF
