"""Pins the oracle (and the model compiler it consumes) to the literal golden
values held by the reference's own tests.  Each test names the reference test
it restates; the expected numbers are the ones written in those tests."""

import os

import numpy as np
import pytest

from brax_gb300 import mjcf
from brax_gb300 import system as S
from oracle.pipeline import Oracle, orthogonals, normalize

_PENDULUM = """
<mujoco model="pendulum">
  <compiler inertiafromgeom="true" autolimits="true"/>
  <option gravity="0 0 -9.81" timestep="0.001"/>
  <worldbody>
    <body name="body1" pos="0 0 0">
      <joint axis="1 0 0" name="hinge1" pos="0 0 0" type="hinge"/>
      <geom name="sphere1" pos="0 0.5 0" size=".15" mass="1" type="sphere"/>
    </body>
  </worldbody>
  <actuator>%s</actuator>
</mujoco>"""


def test_actuator_motor_tau():
  # brax/actuator_test.py:57-60: gear 150 motor, tau = 0.5*9.81
  sys = mjcf.loads(_PENDULUM % '<motor ctrllimited="true" ctrlrange="-100 100" '
                   'joint="hinge1" gear="150"/>')
  o = Oracle(sys, np.float32)
  act = np.array([[1.0 / 150.0 * 0.5 * 9.81]], np.float32)
  tau = o.to_tau(act, np.zeros((1, 1), np.float32), np.zeros((1, 1), np.float32))
  np.testing.assert_array_almost_equal(tau, [[0.5 * 9.81]], 5)


def test_actuator_force_limit():
  # brax/actuator_test.py:114-118: forcerange (-2.5, 3.1), gear 10
  sys = mjcf.loads(_PENDULUM % '<position forcerange="-2.5 3.1" joint="hinge1" '
                   'kp="10" gear="10"/>')
  o = Oracle(sys, np.float32)
  z = np.zeros((1, 1), np.float32)
  for act, lim in [(1000, 3.1), (-1000, -2.5)]:
    tau = o.to_tau(np.array([[act]], np.float32), z, z)
    assert tau[0, 0] == np.float32(lim) * np.float32(10)


def test_pendulum_position_actuator_holds():
  # brax/actuator_test.py:70-78: a position actuator at the target exerts 0
  sys = mjcf.loads(_PENDULUM % '<position ctrllimited="false" joint="hinge1" kp="10"/>')
  o = Oracle(sys, np.float64)
  th = np.pi / 2
  tau = o.to_tau(np.array([[th]]), np.array([[th]]), np.zeros((1, 1)))
  np.testing.assert_array_almost_equal(tau, [[0.0]], 5)


def _ant(ref_path):
  return mjcf.load(os.path.join(ref_path, 'brax/envs/assets/ant.xml'))


def test_ant_init_q(ref_path):
  # brax/kinematics_test.py:69-75
  sys = _ant(ref_path)
  np.testing.assert_almost_equal(
      sys.init_q, np.array([0, 0, 0.55, 1, 0, 0, 0, 0, 1, 0, -1, 0, -1, 0, 1]), 7)


def test_ant_scan_levels(ref_path):
  # brax/scan_test.py:26-66: three levels with these q / qd index sets
  from oracle.pipeline import static
  sys = _ant(ref_path)
  st = static(sys)
  assert sys.link_parents == (-1, 0, 1, 0, 3, 0, 5, 0, 7)
  assert len(st.levels) == 3
  qs = [sum([list(range(st.qadr[i], st.qadr[i] + S.Q_WIDTHS[sys.link_types[i]]))
             for i in lvl], []) for lvl in st.levels]
  ds = [sum([list(range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[sys.link_types[i]]))
             for i in lvl], []) for lvl in st.levels]
  assert qs == [[0, 1, 2, 3, 4, 5, 6], [7, 9, 11, 13], [8, 10, 12, 14]]
  assert ds == [[0, 1, 2, 3, 4, 5], [6, 8, 10, 12], [7, 9, 11, 13]]
  # carry = index + ancestor indices (scan_test.py:44-57)
  carry = []
  for i in range(sys.num_links()):
    j, acc = i, 0
    while j >= 0:
      acc, j = acc + j, sys.link_parents[j]
    carry.append(acc)
  assert carry == [0, 1, 3, 3, 7, 5, 11, 7, 15]


@pytest.mark.parametrize('dtype', [np.float32, np.float64])
def test_ant_sphere_plane_contact(ref_path, dtype):
  # brax/contact_test.py:29-44: all four feet just touch the floor
  sys = _ant(ref_path)
  o = Oracle(sys, dtype)
  q = np.array([[0, 0, 0.556008, 1, 0, 0, 0, 0, 1, 0, 1, 0, 1, 0, 1]], dtype)
  xp, xr, _, _ = o.kinematics(q, np.zeros((1, sys.qd_size()), dtype))
  dist, pos, frame = o.contacts(xp, xr)
  assert dist.shape[1] == 4
  np.testing.assert_array_almost_equal(pos[0, 0], [0.61612, 0.61612, 0])
  np.testing.assert_array_almost_equal(frame[0, 0, 0], [0, 0, 1])
  np.testing.assert_array_almost_equal(dist[0, 0], 0)
  np.testing.assert_array_almost_equal(sys.contacts.friction[0, 0], 1)
  np.testing.assert_array_almost_equal(sys.contacts.elasticity[0], 0)
  assert (sys.contacts.link_a[0], sys.contacts.link_b[0]) == (-1, 2)


_TWO_SPHERES = """
<mujoco model="two_spheres">
  <custom>
    <numeric data="0.2" name="elasticity"/>
    <tuple name="elasticity">
      <element objtype="geom" objname="sphere1" prm="0.1"/>
    </tuple>
  </custom>
  <worldbody>
    <body name="body1" pos="0 0 0">
      <joint name="free1" type="free"/>
      <geom name="sphere1" size="0.2" type="sphere"/>
    </body>
    <body name="body2" pos="0 0 0">
      <joint name="free2" type="free"/>
      <geom name="sphere2" pos="0 0.3 0" size="0.11" type="sphere"/>
    </body>
  </worldbody>
</mujoco>"""


def test_sphere_sphere_contact():
  # brax/contact_test.py:67-75
  sys = mjcf.loads(_TWO_SPHERES)
  o = Oracle(sys, np.float64)
  q = sys.init_q[None]
  xp, xr, _, _ = o.kinematics(q, np.zeros((1, sys.qd_size())))
  dist, pos, frame = o.contacts(xp, xr)
  np.testing.assert_array_almost_equal(dist[0, 0], -0.01)
  np.testing.assert_array_almost_equal(pos[0, 0], [0.0, 0.195, 0.0])
  np.testing.assert_array_almost_equal(frame[0, 0, 0], [0, 1.0, 0.0])
  np.testing.assert_array_almost_equal(sys.contacts.elasticity[0], 0.15)


def test_pair_filter_counts(ref_path):
  # brax/contact_test.py:116-126
  s1 = mjcf.load(os.path.join(ref_path, 'brax/test_data/world_self_collision.xml'))
  assert s1.contacts.n == 13
  s2 = mjcf.load(os.path.join(ref_path, 'brax/test_data/world_fromto.xml'))
  assert s2.contacts.n == 1


def test_inv_approximate():
  # brax/math_test.py:38-46: 100 Newton-Schulz iterations from zero -> inverse
  rng = np.random.default_rng(0)
  for _ in range(5):
    x = rng.normal(size=(4, 4))
    x = np.eye(4) * 0.001 + x @ x.T
    o = Oracle(mjcf.load_asset('chain3'), np.float64)
    xi = o.inv_approximate(x[None], np.zeros((1, 4, 4)), 100)[0]
    # decimal 6 relative to the inverse's scale
    np.testing.assert_array_almost_equal(xi / np.abs(np.linalg.inv(x)).max(),
                                         np.linalg.inv(x) / np.abs(np.linalg.inv(x)).max(), 6)


def test_orthogonals():
  # brax/math_test.py:72-82
  rng = np.random.default_rng(1)
  a = normalize(rng.normal(size=(100, 3)))
  b, c = orthogonals(a)
  np.testing.assert_almost_equal(np.linalg.norm(b, axis=-1), 1)
  np.testing.assert_almost_equal(np.linalg.norm(c, axis=-1), 1)
  for u, v in [(a, b), (b, c), (a, c)]:
    assert np.abs(np.sum(u * v, -1)).max() < 1e-6


_TRIPLE = """
<mujoco model="pendulum">
  <compiler inertiafromgeom="true"/>
  <option gravity="0 0 -9.81" timestep="0.02"/>
  <default><geom contype="0" conaffinity="0"/></default>
  <worldbody>
    <body name="body1" pos="0 0 0">
      <joint axis="1 0 0" name="hinge1" type="hinge"/>
      <geom name="sphere1" pos="0 0.5 0" size=".15" mass="1" type="sphere"/>
      <body name="body2" pos="0 0.5 0">
        <joint axis="1 0 0" name="hinge2" type="hinge"/>
        <geom name="sphere2" pos="0 0.5 0" size=".15" mass="1" type="sphere"/>
        <body name="body3" pos="0 0.5 0">
          <joint axis="1 0 0" name="hinge3" type="hinge"/>
          <geom name="sphere3" pos="0 0.5 0" size=".15" mass="1" type="sphere"/>
        </body>
      </body>
    </body>
  </worldbody>
  <actuator>
    <motor ctrllimited="true" ctrlrange="-100 100" joint="hinge1" gear="150"/>
    <motor ctrllimited="true" ctrlrange="-100 100" joint="hinge2" gear="150"/>
    <motor ctrllimited="true" ctrlrange="-100 100" joint="hinge3" gear="150"/>
  </actuator>
</mujoco>"""


def test_triple_pendulum_rest():
  # brax/actuator_test.py:134-151: hanging straight down with zero action
  sys = mjcf.loads(_TRIPLE)
  for dtype in (np.float32, np.float64):
    o = Oracle(sys, dtype)
    q = np.array([[np.pi / 2, 0.0, 0.0]], dtype)
    s = o.init(q, np.zeros((1, 3), dtype))
    s = o.step(s, np.zeros((1, 3), dtype))
    np.testing.assert_array_almost_equal(s.q, q, 2)
    np.testing.assert_array_almost_equal(s.qd, np.zeros_like(s.qd), 2)


def test_ns_matches_cholesky_inverse():
  # the Newton-Schulz warm start converges to the exact SPD inverse
  sys = mjcf.load_asset('quadruped')
  o = Oracle(sys, np.float64)
  rng = np.random.default_rng(3)
  q = sys.init_q + rng.uniform(-0.1, 0.1, (8, sys.q_size()))
  s = o.init(q, 0.1 * rng.normal(size=(8, sys.qd_size())))
  for _ in range(3):
    s = o.step(s, rng.uniform(-1, 1, (8, sys.act_size())))
  exact = o.spd_inverse(s.mass_mx)
  # NS stops once every residual entry is <= 1e-8 (safe_norm returns 0 there)
  np.testing.assert_allclose(s.mass_mx_inv, exact, rtol=1e-6, atol=1e-7)


def test_fp32_vs_fp64_single_step():
  # FP32 restatement stays within 1e-5 (relative) of FP64 for one step
  for name in ('chain3', 'quadruped', 'humanoid_like'):
    sys = mjcf.load_asset(name)
    rng = np.random.default_rng(0)
    B = 32
    q = sys.init_q + rng.uniform(-0.1, 0.1, (B, sys.q_size()))
    qd = 0.1 * rng.normal(size=(B, sys.qd_size()))
    act = rng.uniform(-1, 1, (B, sys.act_size()))
    o64, o32 = Oracle(sys, np.float64), Oracle(sys, np.float32)
    s64 = o64.step(o64.init(q, qd), act)
    s32 = o32.step(o32.init(q.astype(np.float32), qd.astype(np.float32)),
                   act.astype(np.float32))
    for a, b in ((s32.q, s64.q), (s32.qd, s64.qd)):
      err = np.abs(a - b).max(-1) / np.maximum(np.abs(b).max(-1), 1.0)
      assert np.median(err) < 1e-5, (name, err)


def test_humanoid_newton_schulz_loses_the_inverse():
  """On the humanoid-like workload (gear-100 motors on light limbs, dt 3 ms)
  one step moves M far relative to its smallest eigenvalues (~0.009), the
  reference's Newton-Schulz update (K = 20, math.py:278-305) starts from a
  residual > 1, resets, and its acceptance rule (err starts at 1) then never
  accepts an iterate: mass_mx_inv stops being an inverse.  The exact-inverse
  (Cholesky) mode does not reproduce this, by design; the quadruped stays in
  the converged regime, where both modes agree."""
  from tests.parity_util import actions, seeded_inputs
  sys = mjcf.load_asset('humanoid_like')
  o = Oracle(sys, np.float64)
  q, qd = seeded_inputs(sys, 16, 3)
  s = o.init(q, qd)
  rng = np.random.default_rng(4)
  for _ in range(3):
    s = o.step(s, actions(sys, 16, rng))
  resid = np.linalg.norm(np.eye(sys.qd_size()) - s.mass_mx @ s.mass_mx_inv, axis=(1, 2))
  assert (resid > 1).mean() > 0.5
  sys_q = mjcf.load_asset('quadruped')
  oq = Oracle(sys_q, np.float64)
  q, qd = seeded_inputs(sys_q, 16, 3)
  s = oq.init(q, qd)
  for _ in range(10):
    s = oq.step(s, actions(sys_q, 16, rng))
  resid = np.linalg.norm(np.eye(sys_q.qd_size()) - s.mass_mx @ s.mass_mx_inv, axis=(1, 2))
  assert resid.max() < 1e-6


def test_plane_box_manifold():
  """The restated mjx plane-box manifold: a box resting face-down on the plane
  (every bottom vertex below it) gets three distinct contact points, the
  corners a, b (diagonally opposite a) and c; the fourth choice ties with a
  (equal distances of a and the last corner from the edge bc, first wins) and
  its slot is inactive (dist 1).  A box well above the plane (beyond the 1 mm
  skin) has no candidate vertex: the mask shifts every vertex alike, so the
  slots take vertex 0 and the same geometric choices, all above the plane."""
  from oracle.pipeline import _plane_box
  eye = np.broadcast_to(np.eye(3), (1, 3, 3)).copy()
  size = np.array([0.2, 0.15, 0.1])
  zero = np.zeros((1, 3))
  flat = [_plane_box(zero, eye, np.array([[0.0, 0.0, 0.09]]), eye, size, k) for k in range(4)]
  d = np.array([f[0][0] for f in flat])
  np.testing.assert_allclose(d, [-0.01, -0.01, -0.01, 1.0], atol=1e-12)
  pts = np.array([f[1][0] for f in flat[:3]])
  assert len({tuple(np.round(p, 9)) for p in pts}) == 3
  np.testing.assert_allclose(pts[:, 2], -0.005, atol=1e-12)  # midway between the surfaces
  high = [_plane_box(zero, eye, np.array([[0.0, 0.0, 0.5]]), eye, size, k)[0][0] for k in range(4)]
  assert high[0] == pytest.approx(0.4) and min(high) > 0  # vertex 0 at its distance; nothing active
