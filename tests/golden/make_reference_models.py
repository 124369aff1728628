"""Writes tests/golden/reference_models.json: the System that brax_gb300.mjcf
compiles from each of the reference's environment models
(brax/envs/assets/*.xml), as JSON (brax_gb300.system.to_json).  The GPU tests
run these compiled models, which need no reference checkout at run time.

Usage: python tests/golden/make_reference_models.py <reference checkout>
(or with $BRAXG_REFERENCE set to the checkout).
"""

import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from brax_gb300 import mjcf  # noqa: E402
from brax_gb300 import system as S  # noqa: E402


def main():
  ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('BRAXG_REFERENCE')
  if not ref or not os.path.isdir(os.path.join(ref, 'brax', 'envs', 'assets')):
    sys.exit('usage: make_reference_models.py <reference checkout> (brax/envs/assets not found)')
  out = {}
  for path in sorted(glob.glob(os.path.join(ref, 'brax/envs/assets/*.xml'))):
    name = os.path.splitext(os.path.basename(path))[0]
    out[name] = json.loads(S.to_json(mjcf.load(path)))
  with open(os.path.join(HERE, 'reference_models.json'), 'w') as f:
    json.dump(out, f, separators=(',', ':'))
  print(f'{len(out)} models: {", ".join(out)}')


if __name__ == '__main__':
  main()
