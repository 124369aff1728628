"""Per-env System parameters (braxg_options.randomization; brax's
DomainRandomizationVmapWrapper, brax/envs/wrappers/training.py:223-260):

* overrides equal to the model's values give the unrandomised result bit for
  bit;
* envs with different contact friction, actuator gains, link masses and
  inertias, dof damping or armature match, over one pipeline step, the
  oracle run on a System copy carrying those values, under the single-step
  bar of tests/test_gpu_bench_parity.py (parity_util.oracle_check: p99
  against the FP32 oracle within 1e-5 over the envs FP32 determines to
  1e-5, or 1.5x the FP32 oracle's own FP64 error where the values make the
  model ill-conditioned; every env within its rounding envelope);
* the fused env step and pipeline.randomize accept them.
"""

import dataclasses

import numpy as np
import pytest

from tests.parity_util import actions, load, oracle_check, seeded_inputs

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
  sys_ = load('quadruped')
  n = 192
  q, qd = _settled(sys_, n, 83)
  act = actions(sys_, n, np.random.default_rng(84)).astype(np.float32)
  values = [0.5, 1.0, 1.6]  # per group of 64 envs: friction, or a scale of the field
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
  got_q, got_qd = got.q.cpu().numpy(), got.qd.cpu().numpy()
  for g, v in enumerate(values):
    idx = groups == g
    oracle_check(_with(sys_, field, v), q[idx], qd[idx], None, act[idx], 1, True, got_q[idx], got_qd[idx],
                 f'{field}={v}', strict=True)
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
