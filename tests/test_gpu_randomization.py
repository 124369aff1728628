"""Per-env System parameters (braxg_options.randomization; brax's
DomainRandomizationVmapWrapper, brax/envs/wrappers/training.py:223-260):

* overrides equal to the model's values give the unrandomised result bit for
  bit;
* envs with different contact friction / actuator gains match, over one
  pipeline step, the FP64 oracle run on a System copy carrying those values,
  within max(1e-5, 3x the FP32 oracle's own FP64 error) for 99 % of envs
  (harder contacts and stronger actuators make any FP32 evaluation less
  accurate);
* the fused env step and pipeline.randomize accept them.
"""

import dataclasses

import numpy as np
import pytest

from tests.parity_util import actions, load, rel_err, seeded_inputs

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _P():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline
  return pipeline


def _t(x):
  return torch.as_tensor(np.asarray(x, np.float32), device='cuda')


def _settled(sys_, n, seed):
  """Quadruped states after 10 env steps of the FP64 oracle (feet in contact)."""
  from oracle.pipeline import Oracle
  o = Oracle(sys_, np.float64, exact_inverse=True)
  q, qd = seeded_inputs(sys_, n, seed)
  s = o.init(q, qd)
  rng = np.random.default_rng(seed + 1)
  for _ in range(10):
    s = o.env_step(s, actions(sys_, n, rng), 5)
  return s.q.astype(np.float32), s.qd.astype(np.float32)


def test_model_values_change_nothing():
  P = _P()
  sys_ = load('quadruped')
  m = P.model_for(sys_)
  n = 32
  q, qd = seeded_inputs(sys_, n, 81)
  act = _t(actions(sys_, n, np.random.default_rng(82)))
  s = P.init(sys_, _t(q), _t(qd))
  dr = {'friction': np.tile(sys_.contacts.friction[:, 0], (n, 1)),
        'act_gain': np.tile(sys_.actuator.gain, (n, 1)),
        'act_bias_q': np.tile(sys_.actuator.bias_q, (n, 1)),
        'act_bias_qd': np.tile(sys_.actuator.bias_qd, (n, 1)),
        'link_mass': np.tile(sys_.link.inertia.mass, (n, 1)),
        'link_inertia': np.tile(sys_.link.inertia.i[None], (n, 1, 1, 1)),
        'dof_armature': np.tile(sys_.dof.armature, (n, 1)),
        'dof_damping': np.tile(sys_.dof.damping, (n, 1)),
        'dof_stiffness': np.tile(sys_.dof.stiffness, (n, 1))}
  a = P.step(sys_, s, act, n_frames=5, inverse_mode=P.CHOLESKY)
  b = P.step(sys_, s, act, n_frames=5, inverse_mode=P.CHOLESKY, randomization=dr)
  torch.cuda.synchronize()
  for f in ('q', 'qd', 'mass_mx_inv'):
    torch.testing.assert_close(getattr(a, f), getattr(b, f), rtol=0, atol=0)
  assert m.ncon == sys_.contacts.n


def _with(sys_, field, v):
  """A System copy carrying the value that group's envs get."""
  if field == 'friction':
    fr = sys_.contacts.friction.copy()
    fr[:, 0] = v
    return dataclasses.replace(sys_, contacts=dataclasses.replace(sys_.contacts, friction=fr))
  if field == 'act_gain':
    return dataclasses.replace(sys_, actuator=dataclasses.replace(sys_.actuator, gain=sys_.actuator.gain * v))
  if field == 'link_mass':  # mass and inertia scaled together
    ine = sys_.link.inertia
    ine = dataclasses.replace(ine, mass=ine.mass * v, i=ine.i * v)
    return dataclasses.replace(sys_, link=dataclasses.replace(sys_.link, inertia=ine))
  if field == 'dof_damping':
    return dataclasses.replace(sys_, dof=dataclasses.replace(sys_.dof, damping=sys_.dof.damping * v))
  if field == 'dof_armature':
    return dataclasses.replace(sys_, dof=dataclasses.replace(sys_.dof, armature=sys_.dof.armature + 0.05 * v))
  raise ValueError(field)


def _dr_values(sys_, field, groups, values):
  if field == 'friction':
    return {field: np.stack([np.full(sys_.contacts.n, values[g], np.float32) for g in groups])}
  if field == 'act_gain':
    return {field: np.stack([(sys_.actuator.gain * values[g]).astype(np.float32) for g in groups])}
  if field == 'link_mass':
    return {'link_mass': np.stack([(sys_.link.inertia.mass * values[g]).astype(np.float32) for g in groups]),
            'link_inertia': np.stack([(sys_.link.inertia.i * values[g]).astype(np.float32) for g in groups])}
  if field == 'dof_damping':
    return {field: np.stack([(sys_.dof.damping * values[g]).astype(np.float32) for g in groups])}
  return {field: np.stack([(sys_.dof.armature + 0.05 * values[g]).astype(np.float32) for g in groups])}


@pytest.mark.parametrize('field', ['friction', 'act_gain', 'link_mass', 'dof_damping', 'dof_armature'])
def test_per_env_values_match_oracle_with_those_values(field):
  P = _P()
  from oracle.pipeline import Oracle
  sys_ = load('quadruped')
  n = 48
  q, qd = _settled(sys_, n, 83)
  act = actions(sys_, n, np.random.default_rng(84)).astype(np.float32)
  values = [0.5, 1.0, 1.6]  # per group of 16 envs: friction, or a scale of the field
  groups = np.repeat(np.arange(3), n // 3)
  dr = _dr_values(sys_, field, groups, values)
  s = P.init(sys_, _t(q), _t(qd), randomization=dr)
  got = P.step(sys_, s, _t(act), n_frames=1, inverse_mode=P.CHOLESKY, randomization=dr)
  # the same step without the input state's position-term cache (recomputed
  # with the randomised values) gives the same bits
  nocache = P.step(sys_, s.replace(cache=None), _t(act), n_frames=1, inverse_mode=P.CHOLESKY, randomization=dr)
  torch.cuda.synchronize()
  assert (got.status.cpu().numpy() == 0).all()
  torch.testing.assert_close(got.qd, nocache.qd, rtol=0, atol=0)
  for g, v in enumerate(values):
    sys_g = _with(sys_, field, v)
    idx = groups == g
    o32 = Oracle(sys_g, np.float32, exact_inverse=True)
    o64 = Oracle(sys_g, np.float64, exact_inverse=True)
    r32 = o32.step(o32.init(q[idx], qd[idx]), act[idx])
    r64 = o64.step(o64.init(q[idx].astype(np.float64), qd[idx].astype(np.float64)), act[idx].astype(np.float64))
    for f in ('q', 'qd'):
      gf = getattr(got, f).cpu().numpy()[idx]
      e64 = rel_err(gf, getattr(r64, f))
      eo = rel_err(getattr(r32, f), getattr(r64, f))
      print(f'{field}={v} {f}: vs fp64 p99 {np.quantile(e64, 0.99):.2e} | fp32 oracle vs fp64 p99 '
            f'{np.quantile(eo, 0.99):.2e}')
      assert np.quantile(e64, 0.99) <= max(1e-5, 3 * np.quantile(eo, 0.99)), (field, v, f)
      assert e64.max() <= max(1e-3, 3 * eo.max()), (field, v, f)
  # the groups do differ (the overrides took effect)
  qd_out = got.qd.cpu().numpy()
  assert np.abs(qd_out[groups == 0] - qd_out[groups == 2]).max() > 0


def test_env_step_and_randomize_helper():
  P = _P()
  from brax_gb300 import envs
  sys_ = load('quadruped')
  gen = torch.Generator(device='cuda').manual_seed(85)
  dr = P.randomize(sys_, 64, gen, friction_range=(0.6, 1.4), gain_scale_range=(0.8, 1.2))
  assert dr['friction'].shape == (64, sys_.contacts.n) and dr['act_gain'].shape == (64, sys_.act_size())
  env = envs.Locomotion(sys_, randomization=dr)
  st = env.reset(64, generator=gen)
  st = env.step(st, torch.rand(64, sys_.act_size(), device='cuda', generator=gen) * 2 - 1)
  torch.cuda.synchronize()
  assert torch.isfinite(st.obs).all()
