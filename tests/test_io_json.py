"""The trajectory JSON writer (brax/io/json.py) on CPU, with the checks of
the reference's brax/io/json_test.py:27-52 restated for the packaged models:
geoms grouped by link name (the world's ground plane under 'world'), every
geom carrying size, rgba, name, link_idx, pos and rot, one Transform per
frame, and batched (3-D) frames rejected with RuntimeError."""

import json

import numpy as np
import pytest

from brax_gb300 import io_json, mjcf


def _frames(sys, n):
  from oracle.pipeline import Oracle
  o = Oracle(sys, np.float64)
  s = o.init(sys.init_q[None], np.zeros((1, sys.qd_size())))
  out = []
  for _ in range(n):
    s = o.step(s, np.zeros((1, sys.act_size())))
    out.append((s.x_pos[0], s.x_rot[0]))
  return out


def test_dumps_quadruped():
  sys = mjcf.load_asset('quadruped')
  res = json.loads(io_json.dumps(sys, _frames(sys, 3)))
  assert isinstance(res['geoms'], dict)
  owners = {sys.link_names[b - 1] if b > 0 else 'world' for b in sys.geom_bodyid}
  assert sorted(res['geoms']) == sorted(owners)
  assert len(res['geoms']['world']) == 1 and res['geoms']['world'][0]['name'] == 'Plane'
  for name, gs in res['geoms'].items():
    for g in gs:
      for f in ('size', 'rgba', 'name', 'link_idx', 'pos', 'rot'):
        assert f in g
      assert len(g['size']) == 3 and len(g['rgba']) == 4 and len(g['pos']) == 3 and len(g['rot']) == 4
  torso = res['geoms']['torso'][0]
  assert torso['name'] == 'Sphere' and torso['link_idx'] == 0
  assert torso['rgba'] == [0.4, 0.33, 0.26, 1.0]  # the MJCF default grey becomes brax's default
  assert res['opt']['timestep'] == pytest.approx(sys.dt)
  assert res['name'] == 'System' and res['link_names'] == list(sys.link_names)
  assert len(res['states']['x']) == 3
  x = res['states']['x'][0]
  assert x['name'] == 'Transform'
  assert np.asarray(x['pos']).shape == (sys.num_links(), 3)
  assert np.asarray(x['rot']).shape == (sys.num_links(), 4)


def test_dumps_batched_states_raise():
  sys = mjcf.load_asset('chain3')
  (p, r), = _frames(sys, 1)
  with pytest.raises(RuntimeError):
    io_json.dumps(sys, [(np.stack([p, p]), np.stack([r, r]))])


def test_save_roundtrip(tmp_path):
  sys = mjcf.load_asset('chain3')
  path = tmp_path / 'traj.json'
  io_json.save(str(path), sys, _frames(sys, 2))
  res = json.loads(path.read_text())
  assert len(res['states']['x']) == 2 and 'link1' in res['geoms']
