"""Synthetic workload models and reset distributions.

* ``chain(n)``: an n-link planar chain of capsules (length 0.5 m, radius
  0.05 m, 1 kg each) on hinges about y with damping 0.1, hanging from the
  world; only the last link collides, with a ground plane placed so that it
  just touches the plane when the chain hangs straight.  ``chain(3)`` without
  the plane is the packaged ``chain3`` model.
* ``uneven_mix(total, seed)``: the uneven batch of 60 % chains with link
  counts uniform in 2..32, 25 % quadrupeds and 15 % humanoid-like models.
* ``reset(sys, n, rng)`` / ``actions(sys, n, rng)``: the seeded reset and
  action distributions of each family.
"""

from __future__ import annotations

import functools

import numpy as np

from brax_gb300 import mjcf
from brax_gb300.system import System

LINK_LENGTH = 0.5
LINK_RADIUS = 0.05


def chain_xml(n_links: int) -> str:
  if n_links < 1:
    raise ValueError('a chain needs at least one link')
  floor_z = -(LINK_LENGTH * n_links + LINK_RADIUS) + 0.02
  lines = [
      f'<mujoco model="chain{n_links}">',
      '  <compiler angle="radian" inertiafromgeom="true"/>',
      '  <option gravity="0 0 -9.81" timestep="0.01" iterations="4"/>',
      '  <custom><numeric name="solver_maxls" data="15"/></custom>',
      '  <default>',
      '    <joint type="hinge" axis="0 1 0" damping="0.1"/>',
      f'    <geom type="capsule" size="{LINK_RADIUS}" mass="1" contype="0" conaffinity="0"/>',
      '    <motor ctrllimited="true" ctrlrange="-1 1" gear="10"/>',
      '  </default>',
      '  <worldbody>',
      f'    <geom name="floor" type="plane" size="40 40 40" pos="0 0 {floor_z:.6f}" '
      'contype="0" conaffinity="1"/>',
  ]
  indent = '    '
  for i in range(n_links):
    pos = '0 0 0' if i == 0 else f'0 0 {-LINK_LENGTH}'
    lines.append(f'{indent}<body name="link{i + 1}" pos="{pos}">')
    lines.append(f'{indent}  <joint name="hinge{i + 1}"/>')
    collide = ' contype="1"' if i == n_links - 1 else ''
    lines.append(f'{indent}  <geom name="cap{i + 1}" fromto="0 0 0 0 0 {-LINK_LENGTH}"{collide}/>')
    indent += '  '
  for i in range(n_links - 1, -1, -1):
    indent = indent[:-2]
    lines.append(f'{indent}</body>')
  lines.append('  </worldbody>')
  lines.append('  <actuator>')
  for i in range(n_links):
    lines.append(f'    <motor joint="hinge{i + 1}"/>')
  lines.append('  </actuator>')
  lines.append('</mujoco>')
  return '\n'.join(lines) + '\n'


@functools.lru_cache(maxsize=None)
def chain(n_links: int) -> System:
  return mjcf.loads(chain_xml(n_links))


@functools.lru_cache(maxsize=None)
def asset(name: str) -> System:
  return mjcf.load_asset(name)


def family(sys: System) -> str:
  name = getattr(sys, 'name', '') or ''
  if name.startswith('chain'):
    return 'chain'
  return name


# pipeline steps per env step of each family (brax/envs/base.py:128-137)
N_FRAMES = {'chain': 1, 'quadruped': 5, 'humanoid_like': 5}


def uneven_mix(total: int = 8192, seed: int = 0):
  """[(System, n_env, n_frames)]: 60 % chains of U{2..32} links (one model per
  link count), 25 % quadrupeds, 15 % humanoid-like, ordered as listed."""
  rng = np.random.default_rng(seed)
  n_quad = int(round(0.25 * total))
  n_hum = int(round(0.15 * total))
  n_chain = total - n_quad - n_hum
  links = rng.integers(2, 33, size=n_chain)
  out = []
  for k in range(2, 33):
    c = int((links == k).sum())
    if c:
      out.append((chain(k), c, N_FRAMES['chain']))
  out.append((asset('quadruped'), n_quad, N_FRAMES['quadruped']))
  out.append((asset('humanoid_like'), n_hum, N_FRAMES['humanoid_like']))
  return out


def reset(sys: System, n: int, rng: np.random.Generator, chain_spread: float = 0.1):
  """Seeded (q, qd) for n envs.  Chains hang close to straight with the last
  link on the plane: q ~ U(-chain_spread, chain_spread) per joint, qd ~
  N(0, 0.1) (the 3-link chain workload spreads its 3 joints over
  U(-pi/4, pi/4); spread that wide, chains of 20+ links whip their free end
  past what the semi-implicit integrator holds at dt 0.01, in the FP64
  restatement as well).  Models with a free root: init_q + U(-0.1, 0.1)
  jitter, qd ~ 0.1 N(0, 1) (brax/envs/ant.py:209-213)."""
  nq, nv = sys.q_size(), sys.qd_size()
  if family(sys) == 'chain':
    q = rng.uniform(-chain_spread, chain_spread, (n, nq))
    qd = rng.normal(0.0, 0.1, (n, nv))
  else:
    q = sys.init_q[None] + rng.uniform(-0.1, 0.1, (n, nq))
    qd = 0.1 * rng.normal(size=(n, nv))
  return q, qd


def actions(sys: System, n: int, rng: np.random.Generator):
  """Actions in the control range: chains zero (the plain 3-link chain
  workload's zero actions: gravity and the plane only), humanoid-like
  N(0, 0.3) clipped to [-1, 1], the others U(-1, 1)."""
  nu = sys.act_size()
  if family(sys) == 'chain':
    return np.zeros((n, nu))
  if family(sys) == 'humanoid_like':
    return np.clip(rng.normal(0.0, 0.3, (n, nu)), -1.0, 1.0)
  return rng.uniform(-1.0, 1.0, (n, nu))
