"""The reference's nested State pytree as views of the flat arrays (CPU).

brax code reads ``state.x.pos``, ``state.xd.vel``, ``state.cinr.transform.rot``,
``state.cinr.i``, ``state.cinr.mass``, ``state.cd.ang``, ``state.cdof.vel`` ...
(brax/generalized/base.py:25-92, brax/base.py:396-412).  pipeline.State keeps
the C ABI's flat device arrays and serves those names as views: no copies, so
a write through a view lands in the state.  Checked here on CPU tensors (the
views are plain torch slicing; no kernel runs).
"""

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from brax_gb300 import _native as N  # noqa: E402
from brax_gb300 import mjcf, pipeline as P  # noqa: E402


def _state(n=3, nl=4, nv=5, full=True):
  g = torch.Generator().manual_seed(0)
  r = lambda *s: torch.randn(*s, generator=g)
  s = P.State(q=r(n, 7), qd=r(n, nv), x_pos=r(n, nl, 3), x_rot=r(n, nl, 4), xd_ang=r(n, nl, 3),
              xd_vel=r(n, nl, 3), mass_mx_inv=r(n, nv, nv), qf_smooth=r(n, nv), qf_constraint=r(n, nv),
              qdd=r(n, nv), status=torch.zeros(n, dtype=torch.int32))
  if full:
    s = s.replace(root_com=r(n, nl, 3), cinr_pos=r(n, nl, 3), cinr_rot=r(n, nl, 4), cinr_i=r(n, nl, 3, 3),
                  cinr_mass=r(n, nl), cd_packed=r(n, nl, 6), cdof_packed=r(n, nv, 6), cdofd_packed=r(n, nv, 6),
                  mass_mx=r(n, nv, nv))
  return s


def test_nested_fields_are_views():
  s = _state()
  assert s.x.pos is s.x_pos and s.x.rot is s.x_rot
  assert s.xd.ang is s.xd_ang and s.xd.vel is s.xd_vel
  assert s.cinr.transform.pos is s.cinr_pos and s.cinr.transform.rot is s.cinr_rot
  assert s.cinr.i is s.cinr_i and s.cinr.mass is s.cinr_mass
  for name in ('cd', 'cdof', 'cdofd'):
    m, packed = getattr(s, name), getattr(s, name + '_packed')
    assert torch.equal(m.ang, packed[..., :3]) and torch.equal(m.vel, packed[..., 3:])
    assert m.ang.data_ptr() == packed.data_ptr()  # a view, not a copy
    m.vel[0, 0, 0] = 42.0
    assert packed[0, 0, 3].item() == 42.0


def test_fields_not_produced_are_none():
  s = _state(full=False)
  assert s.x is not None and s.xd is not None
  assert s.cinr is None and s.cd is None and s.cdof is None and s.cdofd is None
  assert s.contact is None


def test_c_state_binds_the_packed_arrays():
  s = _state()
  c = P._cstate(s)
  assert c.cd == s.cd_packed.data_ptr()
  assert c.cdof == s.cdof_packed.data_ptr()
  assert c.cdofd == s.cdofd_packed.data_ptr()
  assert c.x_pos == s.x_pos.data_ptr()
  assert c.contact_dist is None and c.cache is None
  assert [f for f, _ in N.State._fields_] == list(N.STATE_FIELDS)


def test_contact_pytree_constants():
  """Contact carries brax.base.Contact's names; the per-slot constants are the
  model's, broadcast over envs (link_idx -1 is the world body)."""
  sys = mjcf.load_asset('quadruped')

  class _M:  # the two attributes _contact reads from a Model
    ncon = sys.contacts.n

  _M.sys = sys
  n, k = 2, sys.contacts.n
  s = _state(n=n).replace(contact_dist=torch.zeros(n, k), contact_pos=torch.zeros(n, k, 3),
                          contact_frame=torch.zeros(n, k, 3, 3))
  c = P._contact(_M, s)
  assert c.dist is s.contact_dist and c.frame.shape == (n, k, 3, 3)
  assert c.friction.shape == (n, k, 5) and c.solimp.shape == (n, k, 5) and c.solref.shape == (n, k, 2)
  np.testing.assert_array_equal(c.link_idx[0][1].numpy(), sys.contacts.link_a)
  np.testing.assert_array_equal(c.link_idx[1][0].numpy(), sys.contacts.link_b)
  np.testing.assert_array_equal(c.geom[0, :, 0].numpy(), sys.contacts.geom1)
  assert (c.link_idx[0] == -1).all()  # every quadruped contact is against the world plane
  np.testing.assert_allclose(c.elasticity[0].numpy(), sys.contacts.elasticity)


def test_bare_state_carries_only_q_and_qd():
  q, qd = torch.randn(3, 7), torch.randn(3, 5, dtype=torch.float64)
  s = P.bare_state(q, qd)
  assert s.q.dtype == torch.float32 and s.qd.dtype == torch.float32
  assert torch.equal(s.qd, qd.float())
  # every other field the C ABI reads is a null pointer
  cs = P._cstate(s)
  for f in N.STATE_FIELDS:
    if f not in ('q', 'qd'):
      assert getattr(cs, f) is None, f
  assert s.x is None and s.cache is None
  with pytest.raises(ValueError):
    P.bare_state(q, torch.randn(4, 5))
