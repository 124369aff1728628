"""System config and trajectory as JSON for brax's viewer (brax/io/json.py).

Writes the document ``brax.io.json.dumps`` writes: the encoded System fields
the viewer reads (``opt.timestep``, ``link_names``, the class name), the geoms
grouped by link name (type name, link index, pos, rot, rgba, size; the
default MJCF grey becomes brax's default colour) and ``states.x``, one
Transform (pos [nl, 3], rot [nl, 4]) per frame.  Frames come from the
structure-of-arrays state of this package: one env's ``x_pos`` / ``x_rot``
per frame (torch tensors or numpy arrays), e.g. a rollout's per-step outputs
or ``pipeline.State`` objects.
"""

from __future__ import annotations

import json
import math
from typing import Iterable, List, Sequence, Text

import numpy as np

from brax_gb300 import system as S

# brax/io/json.py:47-55
_GEOM_TYPE_NAMES = {S.GEOM_PLANE: 'Plane', S.GEOM_HFIELD: 'HeightMap', S.GEOM_SPHERE: 'Sphere',
                    S.GEOM_CAPSULE: 'Capsule', S.GEOM_CYLINDER: 'Cylinder', S.GEOM_BOX: 'Box',
                    S.GEOM_MESH: 'Mesh'}
_MJCF_DEFAULT_RGBA = (0.5, 0.5, 0.5, 1.0)
_BRAX_DEFAULT_RGBA = [0.4, 0.33, 0.26, 1.0]


def _num(v):
  """Floats as JSON numbers, non-finite ones as strings (brax/io/json.py:75-76)."""
  v = float(v)
  return str(v) if (math.isnan(v) or math.isinf(v)) else v


def _arr(a) -> list:
  a = np.asarray(a.detach().cpu() if hasattr(a, 'detach') else a, dtype=np.float64)
  if a.ndim == 0:
    return _num(a)
  return [_arr(x) for x in a]


def _frame(x_pos, x_rot) -> dict:
  p, r = np.asarray(_as_np(x_pos)), np.asarray(_as_np(x_rot))
  if p.ndim != 2 or r.ndim != 2:
    raise RuntimeError(
        'Expected state.x position and rotation to have 2 shape dimensions but '
        f'received len(pos.shape)={p.ndim} and len(rot.shape)={r.ndim}')
  return {'pos': _arr(p), 'rot': _arr(r), 'name': 'Transform'}


def _as_np(a):
  return a.detach().cpu().numpy() if hasattr(a, 'detach') else np.asarray(a)


def frames_of(states: Iterable) -> List[dict]:
  """One Transform per state: objects with ``x_pos`` / ``x_rot`` of ONE env,
  or (x_pos, x_rot) pairs."""
  out = []
  for st in states:
    if isinstance(st, (tuple, list)):
      out.append(_frame(st[0], st[1]))
    else:
      out.append(_frame(st.x_pos, st.x_rot))
  return out


def dumps(sys: S.System, states: Sequence) -> Text:
  """brax/io/json.py:93-157 for this package's System and states."""
  frames = frames_of(states)
  link_names = [n or f'link {i}' for i, n in enumerate(sys.link_names)] + ['world']
  rgba_all = sys.geom_rgba if sys.geom_rgba is not None else np.tile(_MJCF_DEFAULT_RGBA,
                                                                     (len(sys.geom_type), 1))
  geoms = {}
  for gid in range(len(sys.geom_type)):
    gtype = int(sys.geom_type[gid])
    if gtype == S.GEOM_MESH:
      raise NotImplementedError('mesh geoms are not compiled by this package')
    link_idx = int(sys.geom_bodyid[gid]) - 1
    rgba = np.asarray(rgba_all[gid], dtype=np.float64)
    if np.array_equal(rgba, _MJCF_DEFAULT_RGBA):
      rgba = np.asarray(_BRAX_DEFAULT_RGBA)
    geom = {'name': _GEOM_TYPE_NAMES.get(gtype, str(gtype)), 'link_idx': link_idx,
            'pos': _arr(sys.geom_pos[gid]), 'rot': _arr(sys.geom_quat[gid]), 'rgba': _arr(rgba),
            'size': _arr(sys.geom_size[gid])}
    geoms.setdefault(link_names[link_idx], []).append(geom)
  d = {'opt': {'timestep': _num(sys.dt), 'name': 'Option'}, 'link_names': list(sys.link_names),
       'name': 'System', 'geoms': geoms, 'states': {'x': frames}}
  return json.dumps(d)


def save(path: str, sys: S.System, states: Sequence):
  """Saves a system config and trajectory as json (brax/io/json.py:160-163)."""
  with open(path, 'w') as f:
    f.write(dumps(sys, states))
