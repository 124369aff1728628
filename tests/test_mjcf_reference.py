"""The MJCF compiler on the reference's own fixture models, against the
literal values its loader tests hold (brax/io/mjcf_test.py), plus every
envs/assets model compiling.  Skips where the reference checkout (its XML
fixtures) is absent."""

import glob
import os

import numpy as np
import pytest

from brax_gb300 import mjcf

close = np.testing.assert_array_almost_equal


def _fixture(ref_path, name):
  """test_utils.load_fixture: test_data first, then envs/assets."""
  p = os.path.join(ref_path, 'brax/test_data', name)
  if not os.path.exists(p):
    p = os.path.join(ref_path, 'brax/envs/assets', name)
  return mjcf.load(p)


def test_load_pendulum(ref_path):
  # mjcf_test.py:29-54
  sys = _fixture(ref_path, 'triple_pendulum.xml')
  close(sys.gravity, [0, 0, -9.81])
  assert list(sys.link_names) == ['body1', 'body2', 'body3']
  close(sys.link.transform.pos, [[0, 0, 0], [0, 0.5, 0], [0, 0.5, 0]])
  close(sys.link.transform.rot, [[1, 0, 0, 0]] * 3)
  close(sys.link.inertia.i, np.tile(np.eye(3), (3, 1, 1)) * 0.009)
  close(sys.link.inertia.transform.pos, [[0, 0.5, 0]] * 3)
  close(sys.link.inertia.mass, [1, 1, 1])
  assert sys.link_types == '111'
  assert tuple(sys.link_parents) == (-1, 0, 1)


def test_load_ant(ref_path):
  # mjcf_test.py:56-66
  sys = _fixture(ref_path, 'ant.xml')
  assert list(sys.link_names) == ['torso', 'aux_1', '', 'aux_2', '', 'aux_3', '', 'aux_4', '']
  assert sys.link_types == 'f11111111'
  assert tuple(sys.link_parents) == (-1, 0, 1, 0, 3, 0, 5, 0, 7)


def test_load_humanoid(ref_path):
  # mjcf_test.py:68-89
  sys = _fixture(ref_path, 'humanoid.xml')
  assert list(sys.link_names) == ['torso', 'lwaist', 'pelvis', 'right_thigh', 'right_shin', 'left_thigh',
                                  'left_shin', 'right_upper_arm', 'right_lower_arm', 'left_upper_arm',
                                  'left_lower_arm']
  assert sys.link_types == 'f2131312121'


def test_custom_elasticity(ref_path):
  # mjcf_test.py:91-93
  sys = _fixture(ref_path, 'capsule.xml')
  close(sys.elasticity, [0.2, 0.1])


def test_joint_ref_check(ref_path):
  # mjcf_test.py:95-98
  with pytest.raises(NotImplementedError, match='`ref` attribute'):
    _fixture(ref_path, 'nonzero_joint_ref.xml')


def test_world_body_transform(ref_path):
  # mjcf_test.py:100-109
  sys = _fixture(ref_path, 'world_body_transform.xml')
  r = 0.70710677
  close(sys.geom_pos[1], [1.0, 0.0, 0.0])
  close(sys.geom_quat[1], [r, 0.0, r, 0.0], 5)
  close(sys.init_q, [1.245, 0.0, 0.0, 0.5, 0.5, 0.5, -0.5])


def test_load_fluid_box(ref_path):
  # mjcf_test.py:111-114
  sys = _fixture(ref_path, 'fluid_box.xml')
  close(sys.density, 1.2)
  close(sys.viscosity, 0.15)


def test_load_fluid_ellipsoid(ref_path):
  # mjcf_test.py:116-121
  with pytest.raises(NotImplementedError, match='Ellipsoid fluid model not implemented'):
    _fixture(ref_path, 'fluid_ellipsoid.xml')


def test_load_wind(ref_path):
  # mjcf_test.py:123-128
  with pytest.raises(NotImplementedError, match='option.wind is not implemented'):
    _fixture(ref_path, 'fluid_wind.xml')


def test_world_fromto(ref_path):
  # mjcf_test.py:130-133
  _fixture(ref_path, 'world_fromto.xml')


def test_every_env_asset_compiles(ref_path):
  """brax/envs/assets/*.xml: the models the reference's envs run."""
  paths = sorted(glob.glob(os.path.join(ref_path, 'brax/envs/assets/*.xml')))
  assert paths
  for p in paths:
    sys = mjcf.load(p)
    assert sys.q_size() == len(sys.init_q), p
    assert len(sys.link_types) == sys.num_links() == len(sys.link_parents), p
