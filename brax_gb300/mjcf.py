"""MJCF-subset compiler that builds a ``System`` without MuJoCo.

brax builds its System with ``mujoco.MjModel.from_xml_string`` + ``mjx.put_model``
(brax/io/mjcf.py:317-528).  MuJoCo is a compiled third-party package, absent
here, so this module restates the parts of MuJoCo's model compiler that the
generalized pipeline consumes, from MuJoCo's public modelling documentation
and rigid-body geometry:

* brax's body fusing of joint-less bodies (brax/io/mjcf.py:76-98), including
  its quirk of applying the child offset only when the child ``pos`` is
  non-zero;
* default classes, ``childclass``, compiler ``angle`` units, ``euler`` /
  ``axisangle`` / ``quat`` frames and ``fromto`` capsules;
* body inertia from geoms (``inertiafromgeom``): per-geom mass = density x
  volume (or explicit ``mass``), solid-body inertia of sphere / capsule / box /
  cylinder / ellipsoid, parallel-axis combination, principal axes;
* ``body_invweight0`` (mean diagonal of J M^-1 J^T at the body com, translation
  and rotation blocks) and ``dof_invweight0`` (diagonal of M^-1, averaged over
  the dofs of a free joint's translation / rotation) at ``qpos0``;
* contact candidate generation: every geom pair with a collision function that
  passes contype/conaffinity, same-body and parent-child filtering (the world
  body exempt from the parent-child rule) and ``<exclude>``; friction is the
  max of the two geoms, solref/solimp the mean (equal solmix), elasticity the
  mean (brax/contact.py:59);
* brax's custom ``<numeric>`` parameters and their defaults
  (brax/io/mjcf.py:154-233) and ``load_model``'s field mapping
  (brax/io/mjcf.py:317-489).

Only hinge, slide and free joints are accepted, as brax's ``validate_model``
(brax/io/mjcf.py:236-314) requires; unsupported features raise the same
exception types.
"""

from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional
from xml.etree import ElementTree

import numpy as np

from brax_gb300 import system as S

_ASSET_DIR = os.path.join(os.path.dirname(__file__), 'assets')

# --------------------------------------------------------------------------
# small quaternion helpers (w, x, y, z), float64, host-side only
# --------------------------------------------------------------------------


def _qmul(u, v):
  return np.array([
      u[0] * v[0] - u[1] * v[1] - u[2] * v[2] - u[3] * v[3],
      u[0] * v[1] + u[1] * v[0] + u[2] * v[3] - u[3] * v[2],
      u[0] * v[2] - u[1] * v[3] + u[2] * v[0] + u[3] * v[1],
      u[0] * v[3] + u[1] * v[2] - u[2] * v[1] + u[3] * v[0],
  ])


def _qrot(v, q):
  s, u = q[0], q[1:]
  return 2 * np.dot(u, v) * u + (s * s - np.dot(u, u)) * v + 2 * s * np.cross(u, v)


def _qmat(q):
  q = q / np.linalg.norm(q)
  w, x, y, z = q
  return np.array([
      [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
  ])


def _mat2quat(r):
  """Rotation matrix -> unit quaternion (Shepperd's method), w >= 0."""
  tr = np.trace(r)
  if tr > 0:
    s = math.sqrt(tr + 1.0) * 2
    q = [0.25 * s, (r[2, 1] - r[1, 2]) / s, (r[0, 2] - r[2, 0]) / s,
         (r[1, 0] - r[0, 1]) / s]
  elif r[0, 0] > r[1, 1] and r[0, 0] > r[2, 2]:
    s = math.sqrt(1.0 + r[0, 0] - r[1, 1] - r[2, 2]) * 2
    q = [(r[2, 1] - r[1, 2]) / s, 0.25 * s, (r[0, 1] + r[1, 0]) / s,
         (r[0, 2] + r[2, 0]) / s]
  elif r[1, 1] > r[2, 2]:
    s = math.sqrt(1.0 + r[1, 1] - r[0, 0] - r[2, 2]) * 2
    q = [(r[0, 2] - r[2, 0]) / s, (r[0, 1] + r[1, 0]) / s, 0.25 * s,
         (r[1, 2] + r[2, 1]) / s]
  else:
    s = math.sqrt(1.0 + r[2, 2] - r[0, 0] - r[1, 1]) * 2
    q = [(r[1, 0] - r[0, 1]) / s, (r[0, 2] + r[2, 0]) / s,
         (r[1, 2] + r[2, 1]) / s, 0.25 * s]
  q = np.array(q)
  q = q / np.linalg.norm(q)
  return q if q[0] >= 0 else -q


def _axisangle(axis, angle):
  axis = np.asarray(axis, dtype=np.float64)
  n = np.linalg.norm(axis)
  if n < 1e-15:
    return np.array([1.0, 0, 0, 0])
  axis = axis / n
  return np.concatenate([[math.cos(angle / 2)], axis * math.sin(angle / 2)])


def _euler_xyz(e):
  """Intrinsic x-y'-z'' Euler angles (MuJoCo's default eulerseq)."""
  q = np.array([1.0, 0, 0, 0])
  for k in range(3):
    ax = np.zeros(3)
    ax[k] = 1.0
    q = _qmul(q, _axisangle(ax, e[k]))
  return q


def _quat_z2vec(v):
  """Minimal rotation taking +z onto direction v."""
  v = np.asarray(v, dtype=np.float64)
  n = np.linalg.norm(v)
  if n < 1e-15:
    return np.array([1.0, 0, 0, 0])
  v = v / n
  z = np.array([0.0, 0, 1])
  ax = np.cross(z, v)
  s = np.linalg.norm(ax)
  if s < 1e-14:
    return np.array([1.0, 0, 0, 0]) if v[2] > 0 else np.array([0.0, 1, 0, 0])
  return _axisangle(ax / s, math.atan2(s, v[2]))


# --------------------------------------------------------------------------
# parsing
# --------------------------------------------------------------------------


def _vec(s: Optional[str], n: Optional[int] = None, default=None):
  if s is None:
    return None if default is None else np.array(default, dtype=np.float64)
  v = np.array([float(t) for t in s.split()], dtype=np.float64)
  if n is not None and v.shape[0] < n:
    d = np.array(default if default is not None else [0.0] * n, dtype=np.float64)
    d[: v.shape[0]] = v
    v = d
  return v


@dataclasses.dataclass
class _Elem:
  tag: str
  attrib: Dict[str, str]
  children: List['_Elem']


@dataclasses.dataclass
class _Ctx:
  angle_scale: float
  defaults: Dict[str, Dict[str, Dict[str, str]]]
  autolimits: bool = True


def _read_defaults(root: ElementTree.Element) -> Dict[str, Dict[str, Dict[str, str]]]:
  classes: Dict[str, Dict[str, Dict[str, str]]] = {}

  def walk(elem, name, inherited):
    mine = {k: dict(v) for k, v in inherited.items()}
    for child in elem:
      if child.tag == 'default':
        continue
      mine.setdefault(child.tag, {}).update(child.attrib)
    classes[name] = mine
    for child in elem:
      if child.tag == 'default':
        walk(child, child.attrib.get('class', name), mine)

  for d in root.findall('default'):
    walk(d, d.attrib.get('class', 'main'), {})
  classes.setdefault('main', {})
  return classes


def _resolve(elem: ElementTree.Element, ctx: _Ctx, cls: str) -> Dict[str, str]:
  cls = elem.attrib.get('class', cls)
  if cls not in ctx.defaults:
    raise ValueError(f'unknown default class "{cls}"')
  tag = elem.tag
  if tag == 'freejoint':  # a <freejoint> takes no class defaults
    return dict(elem.attrib)
  base = dict(ctx.defaults[cls].get(tag, {}))
  if tag in ('motor', 'position', 'velocity'):
    base = {**ctx.defaults[cls].get('general', {}), **base}
  base.update(elem.attrib)
  return base


def _frame(attrib: Dict[str, str], ctx: _Ctx):
  pos = _vec(attrib.get('pos'), 3, [0, 0, 0])
  if 'quat' in attrib:
    quat = _vec(attrib['quat'])
    quat = quat / np.linalg.norm(quat)
  elif 'euler' in attrib:
    quat = _euler_xyz(_vec(attrib['euler']) * ctx.angle_scale)
  elif 'axisangle' in attrib:
    aa = _vec(attrib['axisangle'])
    quat = _axisangle(aa[:3], aa[3] * ctx.angle_scale)
  elif 'zaxis' in attrib:
    quat = _quat_z2vec(_vec(attrib['zaxis']))
  else:
    quat = np.array([1.0, 0, 0, 0])
  return pos, quat


def _parse_body(elem: ElementTree.Element, ctx: _Ctx, cls: str) -> _Elem:
  attrib = dict(elem.attrib)
  childcls = elem.attrib.get('childclass', cls)
  children = []
  for child in elem:
    if child.tag in ('body',):
      children.append(_parse_body(child, ctx, childcls))
    elif child.tag in ('geom', 'joint', 'freejoint', 'inertial', 'site'):
      children.append(_Elem(child.tag, _resolve(child, ctx, childcls), []))
  return _Elem('body', attrib, children)


def _fuse_frame(attrib: Dict[str, str], ctx: _Ctx):
  """An element's frame as body fusing reads it: a `quat` attribute as
  written (not normalised: rotating by it scales by its squared norm, as the
  reference's fusing does), other orientation forms as unit quaternions."""
  if 'quat' in attrib:
    return _vec(attrib.get('pos'), 3, [0, 0, 0]), _vec(attrib['quat'])
  return _frame(attrib, ctx)


def _fmt(v) -> str:
  """The fused attributes are written with 6 decimals, as the reference's
  fusing writes them ('%f')."""
  return ' '.join('%f' % float(x) for x in v)


def _offset(e: _Elem, ppos, pquat, ctx: _Ctx):
  """Moves an element into its grandparent's frame (brax/io/mjcf.py:47-73)."""
  if 'fromto' in e.attrib:
    ft = _vec(e.attrib['fromto'])
    a = ppos + _qrot(ft[0:3], pquat)
    b = ppos + _qrot(ft[3:6], pquat)
    e.attrib['fromto'] = _fmt(np.concatenate([a, b]))
    return
  pos, quat = _fuse_frame(e.attrib, ctx)
  pos = ppos + _qrot(pos, pquat)
  quat = _qmul(pquat, quat)
  for k in ('euler', 'axisangle', 'zaxis'):
    e.attrib.pop(k, None)
  e.attrib['pos'] = _fmt(pos)
  e.attrib['quat'] = _fmt(quat)


def _fuse(elem: _Elem, ctx: _Ctx):
  """Fuses joint-less child bodies into their parent (brax/io/mjcf.py:76-98)."""
  for child in list(elem.children):
    _fuse(child, ctx)
    if child.tag != 'body':
      continue
    if any(c.tag in ('joint', 'freejoint') for c in child.children):
      continue
    cpos, cquat = _fuse_frame(child.attrib, ctx)
    for gc in child.children:
      if gc.tag in ('body', 'geom', 'site') and (cpos != 0).any():
        _offset(gc, cpos, cquat, ctx)
      elem.children.append(gc)
    elem.children.remove(child)


# --------------------------------------------------------------------------
# geometry: mass properties
# --------------------------------------------------------------------------


def _geom_frame(g: Dict[str, str], ctx: _Ctx, gtype: int):
  size = _vec(g.get('size'), 3, [0, 0, 0])
  if 'fromto' in g:
    ft = _vec(g['fromto'])
    a, b = ft[0:3], ft[3:6]
    pos = 0.5 * (a + b)
    quat = _quat_z2vec(b - a)
    half = 0.5 * np.linalg.norm(b - a)
    if gtype in (S.GEOM_CAPSULE, S.GEOM_CYLINDER):
      size = np.array([size[0], half, 0.0])
    elif gtype == S.GEOM_BOX:
      size = np.array([size[0], size[0] if size[1] == 0 else size[1], half])
    return pos, quat, size
  pos, quat = _frame(g, ctx)
  return pos, quat, size


def _geom_mass(gtype: int, size: np.ndarray, g: Dict[str, str]):
  """Mass and principal inertia (geom frame) of a solid geom."""
  r = size[0]
  if gtype == S.GEOM_SPHERE:
    vol = 4.0 / 3.0 * math.pi * r ** 3
  elif gtype == S.GEOM_CAPSULE:
    vol = math.pi * r * r * 2 * size[1] + 4.0 / 3.0 * math.pi * r ** 3
  elif gtype == S.GEOM_CYLINDER:
    vol = math.pi * r * r * 2 * size[1]
  elif gtype == S.GEOM_BOX:
    vol = 8 * size[0] * size[1] * size[2]
  elif gtype == S.GEOM_ELLIPSOID:
    vol = 4.0 / 3.0 * math.pi * size[0] * size[1] * size[2]
  else:
    return 0.0, np.zeros(3)
  if 'mass' in g:
    mass = float(g['mass'])
    density = mass / vol if vol > 0 else 0.0
  else:
    density = float(g.get('density', 1000.0))
    mass = density * vol
  if gtype == S.GEOM_SPHERE:
    i = np.full(3, 0.4 * mass * r * r)
  elif gtype == S.GEOM_CAPSULE:
    h = 2 * size[1]
    m_cyl = density * math.pi * r * r * h
    m_sph = density * 4.0 / 3.0 * math.pi * r ** 3
    ixx = (m_cyl * (3 * r * r + h * h) / 12.0
           + m_sph * (0.4 * r * r + 0.25 * h * h + 0.375 * h * r))
    izz = 0.5 * m_cyl * r * r + 0.4 * m_sph * r * r
    i = np.array([ixx, ixx, izz])
  elif gtype == S.GEOM_CYLINDER:
    h = 2 * size[1]
    ixx = mass * (3 * r * r + h * h) / 12.0
    i = np.array([ixx, ixx, 0.5 * mass * r * r])
  elif gtype == S.GEOM_BOX:
    a, b, c = size
    i = mass / 3.0 * np.array([b * b + c * c, a * a + c * c, a * a + b * b])
  else:  # ellipsoid
    a, b, c = size
    i = mass / 5.0 * np.array([b * b + c * c, a * a + c * c, a * a + b * b])
  return mass, i


_GEOM_TYPES = {'plane': S.GEOM_PLANE, 'hfield': S.GEOM_HFIELD,
               'sphere': S.GEOM_SPHERE, 'capsule': S.GEOM_CAPSULE,
               'ellipsoid': S.GEOM_ELLIPSOID, 'cylinder': S.GEOM_CYLINDER,
               'box': S.GEOM_BOX, 'mesh': S.GEOM_MESH}


# --------------------------------------------------------------------------
# compile
# --------------------------------------------------------------------------


@dataclasses.dataclass
class _Body:
  name: str
  parent: int
  pos: np.ndarray
  quat: np.ndarray
  joints: List[Dict[str, str]]
  geoms: List[Dict[str, str]]
  inertial: Optional[Dict[str, str]]


def _flatten(world: _Elem, ctx: _Ctx) -> List[_Body]:
  bodies = [_Body('world', -1, np.zeros(3), np.array([1.0, 0, 0, 0]), [],
                  [c.attrib for c in world.children if c.tag == 'geom'], None)]

  def walk(e: _Elem, parent: int):
    for c in e.children:
      if c.tag != 'body':
        continue
      pos, quat = _frame(c.attrib, ctx)
      joints = []
      for j in c.children:
        if j.tag == 'freejoint':
          joints.append({**j.attrib, 'type': 'free'})
        elif j.tag == 'joint':
          joints.append(j.attrib)
      inertial = next((j.attrib for j in c.children if j.tag == 'inertial'), None)
      idx = len(bodies)
      bodies.append(_Body(c.attrib.get('name', ''), parent, pos, quat,
                          joints, [g.attrib for g in c.children if g.tag == 'geom'],
                          inertial))
      walk(c, idx)

  walk(world, 0)
  return bodies


def _body_inertia(b: _Body, ctx: _Ctx, inertiafromgeom: str):
  """(mass, ipos, iquat, diag inertia) of a body in the body frame."""
  use_geoms = inertiafromgeom == 'true' or (
      inertiafromgeom == 'auto' and b.inertial is None)
  if not use_geoms and b.inertial is not None:
    it = b.inertial
    pos, quat = _frame(it, ctx)
    mass = float(it.get('mass', 0.0))
    if 'fullinertia' in it:
      f = _vec(it['fullinertia'])
      full = np.array([[f[0], f[3], f[4]], [f[3], f[1], f[5]], [f[4], f[5], f[2]]])
      rot = _qmat(quat)
      full = rot @ full @ rot.T
      return _principal(mass, pos, full)
    diag = _vec(it.get('diaginertia'), 3, [0, 0, 0])
    return mass, pos, quat, diag
  mass, com = 0.0, np.zeros(3)
  parts = []
  for g in b.geoms:
    gtype = _GEOM_TYPES[g.get('type', 'sphere')]
    gpos, gquat, size = _geom_frame(g, ctx, gtype)
    m, i = _geom_mass(gtype, size, g)
    if m <= 0:
      continue
    parts.append((m, gpos, _qmat(gquat) @ np.diag(i) @ _qmat(gquat).T))
    mass += m
    com += m * gpos
  if mass <= 0:
    return 0.0, np.zeros(3), np.array([1.0, 0, 0, 0]), np.zeros(3)
  com /= mass
  full = np.zeros((3, 3))
  for m, p, i in parts:
    d = p - com
    full += i + m * (np.dot(d, d) * np.eye(3) - np.outer(d, d))
  return _principal(mass, com, full)


def _principal(mass, com, full):
  w, v = np.linalg.eigh(0.5 * (full + full.T))
  order = np.argsort(-w)  # MuJoCo lists principal moments largest first
  w, v = w[order], v[:, order]
  if np.linalg.det(v) < 0:
    v[:, 2] = -v[:, 2]
  return mass, com, _mat2quat(v), np.maximum(w, 0.0)


def _custom(root: ElementTree.Element, nbody: int, ngeom: int, nq: int,
            geom_names: List[str]):
  """brax custom parameters with defaults (brax/io/mjcf.py:154-233)."""
  default = {
      'ang_damping': (0.0, None), 'vel_damping': (0.0, None),
      'baumgarte_erp': (0.1, None), 'spring_mass_scale': (0.0, None),
      'spring_inertia_scale': (0.0, None), 'joint_scale_pos': (0.5, None),
      'joint_scale_ang': (0.2, None), 'collide_scale': (1.0, None),
      'matrix_inv_iterations': (10, None), 'solver_maxls': (20, None),
      'elasticity': (0.0, 'geom'), 'constraint_stiffness': (2000.0, 'body'),
      'constraint_limit_stiffness': (1000.0, 'body'),
      'constraint_ang_damping': (0.0, 'body'),
      'constraint_vel_damping': (0.0, 'body'),
  }
  for c in root.findall('custom'):
    for n in c.findall('numeric'):
      name = n.attrib['name']
      val = _vec(n.attrib.get('data', '0'))
      typ = default[name][1] if name in default else None
      default[name] = (val, typ)
  out = {}
  for name, (val, typ) in default.items():
    val = np.atleast_1d(np.array(val, dtype=np.float64))
    size = {'body': nbody - 1, 'geom': ngeom}.get(typ, val.shape[-1])
    if val.shape[-1] != size and val.shape[-1] > 1:
      raise ValueError(f'"{name}" custom arg needed {size} values for the '
                       f'"{typ}" type, but got {val.shape[-1]} values.')
    if val.shape[-1] != size:
      val = np.repeat(val, size)
    out[name] = val if typ else (val[0] if val.shape[0] == 1 else val)
  # tuple overrides for geom-typed parameters (brax/io/mjcf.py:201-229)
  for c in root.findall('custom'):
    for t in c.findall('tuple'):
      name = t.attrib['name']
      elems = t.findall('element')
      if any(e.attrib.get('objtype') != 'geom' for e in elems):
        raise NotImplementedError(
            f'Custom tuple "{name}" with a non-geom objtype is not supported.')
      if name in default and default[name][1] != 'geom':
        raise ValueError(f'Custom tuple "{name}" is expected to be associated '
                         f'with the {default[name][1]} objtype.')
      base = np.atleast_1d(np.array(default.get(name, (0.0, None))[0], np.float64))
      arr = np.repeat(base[:1], ngeom)
      for e in elems:
        arr[geom_names.index(e.attrib['objname'])] = float(e.attrib['prm'])
      out[name] = arr
  if 'init_qpos' in out and np.atleast_1d(out['init_qpos']).shape[0] != nq:
    size = np.atleast_1d(out['init_qpos']).shape[0]
    raise ValueError(f'init_qpos had length {size} but expected length {nq}.')
  return out


def loads(xml: str, name: str = '') -> S.System:
  """Compiles an MJCF string into a System (brax.io.mjcf.loads)."""
  root = ElementTree.fromstring(xml)
  comp = root.find('compiler')
  comp_attr = comp.attrib if comp is not None else {}
  angle = comp_attr.get('angle', 'degree')
  ctx = _Ctx(angle_scale=(math.pi / 180.0) if angle == 'degree' else 1.0,
             defaults=_read_defaults(root),
             autolimits=comp_attr.get('autolimits', 'true') == 'true')
  inertiafromgeom = comp_attr.get('inertiafromgeom', 'auto')

  opt = root.find('option')
  oa = opt.attrib if opt is not None else {}
  if oa.get('integrator', 'Euler') not in ('Euler',):
    raise NotImplementedError('Only euler integration is supported.')
  if oa.get('cone', 'pyramidal') != 'pyramidal':
    raise NotImplementedError('Only pyramidal cone friction is supported.')
  if float(oa.get('impratio', 1)) != 1:
    raise NotImplementedError('Only impratio=1 is supported.')
  if 'wind' in oa and np.any(_vec(oa['wind'])):
    raise NotImplementedError('option.wind is not implemented.')
  dt = float(oa.get('timestep', 0.002))
  gravity = _vec(oa.get('gravity'), 3, [0, 0, -9.81])
  iterations = int(oa.get('iterations', 100))
  viscosity = float(oa.get('viscosity', 0.0))
  density = float(oa.get('density', 0.0))

  wb = root.find('worldbody')
  world = _Elem('worldbody', {}, [])
  for child in wb:
    if child.tag == 'body':
      world.children.append(_parse_body(child, ctx, 'main'))
    elif child.tag in ('geom', 'site'):
      world.children.append(_Elem(child.tag, _resolve(child, ctx, 'main'), []))
  _fuse(world, ctx)
  bodies = _flatten(world, ctx)
  nbody = len(bodies)

  # --- joints -> link types, dofs -----------------------------------------
  link_types, jnts = '', []
  # qpos0 of the non-free joints (brax/io/mjcf.py:266-271 checks it before
  # the joint stacks)
  if any(j.get('type', 'hinge') != 'free' and float(j.get('ref', 0.0)) != 0.0
         for b in bodies[1:] for j in b.joints):
    raise NotImplementedError('The `ref` attribute on joint types is not supported.')
  for bi, b in enumerate(bodies[1:], start=1):
    types = [j.get('type', 'hinge') for j in b.joints]
    if not types:
      raise NotImplementedError(
          f'body "{b.name}" has no joint; only jointed bodies become links')
    if 'ball' in types:
      raise NotImplementedError('ball joints not supported')
    if 'free' in types:
      if len(types) != 1:
        raise RuntimeError('invalid joint stack: cannot stack free joints')
      link_types += 'f'
    else:
      if len(types) > 3:
        raise NotImplementedError('at most 3 stacked joints per body')
      link_types += str(len(types))
    poss = [_vec(j.get('pos'), 3, [0, 0, 0]) for j in b.joints]
    if any((p != poss[0]).any() for p in poss):
      raise RuntimeError('invalid joint stack: only one joint position allowed')
    for j in b.joints:
      jnts.append((bi, j))
  nl = nbody - 1
  link_parents = tuple(b.parent - 1 for b in bodies[1:])
  for i, p in enumerate(link_parents):
    if p >= i:
      raise ValueError('bodies must be listed parents first')

  motions_ang, motions_vel = [], []
  armature, stiffness, damping, lo, hi, solp = [], [], [], [], [], []
  jnt_qadr, jnt_dadr, jnt_names = [], [], []
  any_limited = False
  q0 = []
  qa = da = 0
  for bi, j in jnts:
    typ = j.get('type', 'hinge')
    jnt_names.append(j.get('name', ''))
    jnt_qadr.append(qa)
    jnt_dadr.append(da)
    arm = float(j.get('armature', 0.0))
    damp = float(j.get('damping', 0.0))
    stiff = float(j.get('stiffness', 0.0))
    solref = _vec(j.get('solreflimit'), 2, [0.02, 1.0])
    solimp = _vec(j.get('solimplimit'), 5, [0.9, 0.95, 0.001, 0.5, 2.0])
    if typ == 'free':
      if stiff > 0:
        raise RuntimeError('brax does not support stiffness for free joints')
      motions_ang.append(np.eye(6, 3, -3))
      motions_vel.append(np.eye(6, 3))
      armature += [arm] * 6
      stiffness += [0.0] * 6
      damping += [damp] * 6
      lo += [-np.inf] * 6
      hi += [np.inf] * 6
      solp += [np.concatenate([solref, solimp])] * 6
      b = bodies[bi]
      q0 += list(b.pos) + list(b.quat)
      qa, da = qa + 7, da + 6
      continue
    axis = _vec(j.get('axis'), 3, [0, 0, 1])
    axis = axis / np.linalg.norm(axis)
    rng = _vec(j.get('range'), 2, [0, 0])
    lim = j.get('limited', 'auto')
    limited = lim == 'true' or (lim == 'auto' and ctx.autolimits and 'range' in j
                               and rng[0] < rng[1])
    if typ == 'hinge':
      rng = rng * ctx.angle_scale
      motions_ang.append(axis[None])
      motions_vel.append(np.zeros((1, 3)))
    elif typ == 'slide':
      motions_ang.append(np.zeros((1, 3)))
      motions_vel.append(axis[None])
    else:
      raise RuntimeError(f'invalid joint type: {typ}')
    any_limited |= limited
    armature.append(arm)
    stiffness.append(stiff)
    damping.append(damp)
    lo.append(rng[0] if limited else -np.inf)
    hi.append(rng[1] if limited else np.inf)
    solp.append(np.concatenate([solref, solimp]))
    q0.append(0.0)
    qa, da = qa + 1, da + 1
  nq, nv = qa, da
  dof_ang = np.concatenate(motions_ang) if motions_ang else np.zeros((0, 3))
  dof_vel = np.concatenate(motions_vel) if motions_vel else np.zeros((0, 3))

  # --- links ------------------------------------------------------------
  link_pos = np.array([b.pos for b in bodies[1:]]).reshape(nl, 3)
  link_rot = np.array([b.quat for b in bodies[1:]]).reshape(nl, 4)
  joint_pos = np.array([_vec(b.joints[0].get('pos'), 3, [0, 0, 0])
                        if b.joints[0].get('type') != 'free' else
                        _vec(b.joints[0].get('pos'), 3, [0, 0, 0])
                        for b in bodies[1:]]).reshape(nl, 3)
  mass, ipos, iquat, idiag = [], [], [], []
  for b in bodies[1:]:
    m, p, q, d = _body_inertia(b, ctx, inertiafromgeom)
    mass.append(m)
    ipos.append(p)
    iquat.append(q)
    idiag.append(d)
  mass = np.array(mass).reshape(nl)
  ipos = np.array(ipos).reshape(nl, 3)
  iquat = np.array(iquat).reshape(nl, 4)
  inertia_i = np.array([np.diag(d) for d in idiag]).reshape(nl, 3, 3)
  for i, t in enumerate(link_types):
    if t == 'f':  # brax/io/mjcf.py:414-419
      link_pos[i] = 0.0
      link_rot[i] = np.array([1.0, 0, 0, 0])

  # --- geoms ------------------------------------------------------------
  g_type, g_body, g_pos, g_quat, g_size = [], [], [], [], []
  g_fric, g_sr, g_si, g_ct, g_ca, g_names, g_rgba = [], [], [], [], [], [], []
  for bi, b in enumerate(bodies):
    for g in b.geoms:
      if g.get('fluidshape', 'none') == 'ellipsoid':  # geom_fluid != 0, brax/io/mjcf.py:242-243
        raise NotImplementedError('Ellipsoid fluid model not implemented.')
      gt = _GEOM_TYPES[g.get('type', 'sphere')]
      if gt in (S.GEOM_HFIELD, S.GEOM_MESH, S.GEOM_ELLIPSOID):
        if int(g.get('contype', 1)) | int(g.get('conaffinity', 1)):
          raise NotImplementedError(f'collision geom type {gt} not supported')
      if gt == S.GEOM_CYLINDER:
        gp, gq, sz = _geom_frame(g, ctx, gt)
        if sz[1] > 0.001 and (int(g.get('contype', 1)) | int(g.get('conaffinity', 1))):
          raise NotImplementedError(
              'Cylinders of half-length>0.001 are not supported for collision.')
      gp, gq, sz = _geom_frame(g, ctx, gt)
      g_type.append(gt)
      g_body.append(bi)
      g_pos.append(gp)
      g_quat.append(gq)
      g_size.append(sz)
      g_fric.append(_vec(g.get('friction'), 3, [1.0, 0.005, 0.0001]))
      g_sr.append(_vec(g.get('solref'), 2, [0.02, 1.0]))
      g_si.append(_vec(g.get('solimp'), 5, [0.9, 0.95, 0.001, 0.5, 2.0]))
      g_ct.append(int(g.get('contype', 1)))
      g_ca.append(int(g.get('conaffinity', 1)))
      g_names.append(g.get('name', ''))
      g_rgba.append(_vec(g.get('rgba'), 4, [0.5, 0.5, 0.5, 1.0]))
      if float(g.get('solmix', 1.0)) != 1.0:
        raise NotImplementedError('geom_solmix parameter not supported.')
      if int(g.get('priority', 0)) != 0:
        raise NotImplementedError('geom_priority parameter not supported.')
  ngeom = len(g_type)
  g_type = np.array(g_type, dtype=np.int64)
  g_body = np.array(g_body, dtype=np.int64)
  g_pos = np.array(g_pos).reshape(ngeom, 3)
  g_quat = np.array(g_quat).reshape(ngeom, 4)
  g_size = np.array(g_size).reshape(ngeom, 3)
  g_fric = np.array(g_fric).reshape(ngeom, 3)
  g_sr = np.array(g_sr).reshape(ngeom, 2)
  g_si = np.array(g_si).reshape(ngeom, 5)
  g_ct = np.array(g_ct, dtype=np.int64)
  g_ca = np.array(g_ca, dtype=np.int64)

  custom = _custom(root, nbody, ngeom, nq, g_names)
  elasticity = np.asarray(custom['elasticity'], dtype=np.float64).reshape(ngeom)

  # --- actuators -------------------------------------------------------
  jnt_by_name = {n: k for k, n in enumerate(jnt_names)}
  a_q, a_d, a_cr, a_fr, a_gain, a_gear, a_bq, a_bd = [], [], [], [], [], [], [], []
  act = root.find('actuator')
  for a in (list(act) if act is not None else []):
    attr = _resolve(a, ctx, a.attrib.get('class', 'main'))
    if 'joint' not in attr:
      raise NotImplementedError(
          'Only joint transmission types are supported for actuators.')
    k = jnt_by_name[attr['joint']]
    if jnts[k][1].get('type') == 'free':
      raise NotImplementedError('actuators on free joints are not supported')
    gear = _vec(attr.get('gear'), 6, [1, 0, 0, 0, 0, 0])[0]
    cr = _vec(attr.get('ctrlrange'), 2, [0, 0])
    cl = attr.get('ctrllimited', 'auto')
    ctrllimited = cl == 'true' or (cl == 'auto' and 'ctrlrange' in attr and cr[0] < cr[1])
    fr = _vec(attr.get('forcerange'), 2, [0, 0])
    fl = attr.get('forcelimited', 'auto')
    forcelimited = fl == 'true' or (fl == 'auto' and 'forcerange' in attr and fr[0] < fr[1])
    if a.tag == 'motor':
      gain, bq, bd = 1.0, 0.0, 0.0
    elif a.tag == 'position':
      kp = float(attr.get('kp', 1.0))
      gain, bq, bd = kp, -kp, -float(attr.get('kv', 0.0))
    elif a.tag == 'velocity':
      kv = float(attr.get('kv', 1.0))
      gain, bq, bd = kv, 0.0, -kv
    elif a.tag == 'general':
      if attr.get('gaintype', 'fixed') != 'fixed':
        raise NotImplementedError('Only actuator_gaintype in [0] is supported.')
      bt = attr.get('biastype', 'none')
      if bt not in ('none', 'affine'):
        raise NotImplementedError('Only actuator_biastype in [0, 1] are supported.')
      gp = _vec(attr.get('gainprm'), 3, [1, 0, 0])
      bp = _vec(attr.get('biasprm'), 3, [0, 0, 0])
      gain = gp[0]
      bq, bd = (bp[1], bp[2]) if bt == 'affine' else (0.0, 0.0)
    else:
      raise NotImplementedError(f'actuator type {a.tag} is not supported')
    a_q.append(jnt_qadr[k])
    a_d.append(jnt_dadr[k])
    a_cr.append(cr if ctrllimited else np.array([-np.inf, np.inf]))
    a_fr.append(fr if forcelimited else np.array([-np.inf, np.inf]))
    a_gain.append(gain)
    a_gear.append(gear)
    a_bq.append(bq)
    a_bd.append(bd)
  nu = len(a_q)
  actuator = S.Actuator(
      q_id=np.array(a_q, dtype=np.int64), qd_id=np.array(a_d, dtype=np.int64),
      ctrl_range=np.array(a_cr).reshape(nu, 2),
      force_range=np.array(a_fr).reshape(nu, 2),
      gain=np.array(a_gain), gear=np.array(a_gear),
      bias_q=np.array(a_bq), bias_qd=np.array(a_bd))

  # --- contact candidates -------------------------------------------------
  excludes = set()
  con = root.find('contact')
  if con is not None:
    names = {b.name: i for i, b in enumerate(bodies) if b.name}
    for ex in con.findall('exclude'):
      b1, b2 = names[ex.attrib['body1']], names[ex.attrib['body2']]
      excludes.add((min(b1, b2), max(b1, b2)))
    if con.findall('pair'):
      raise NotImplementedError('explicit <pair> contacts are not supported')
  parent_body = [b.parent for b in bodies]
  pairs = []
  for g1 in range(ngeom):
    for g2 in range(g1 + 1, ngeom):
      b1, b2 = g_body[g1], g_body[g2]
      if b1 == b2:
        continue
      if not ((g_ct[g1] & g_ca[g2]) or (g_ct[g2] & g_ca[g1])):
        continue
      if b1 != 0 and b2 != 0 and (parent_body[b1] == b2 or parent_body[b2] == b1):
        continue
      if (min(b1, b2), max(b1, b2)) in excludes:
        continue
      t1, t2 = g_type[g1], g_type[g2]
      a, b = (g1, g2) if t1 <= t2 else (g2, g1)
      key = (int(g_type[a]), int(g_type[b]))
      if key not in S.CON_KIND:
        raise NotImplementedError(f'no collision function for geom types {key}')
      pairs.append((S.CON_KIND[key], a, b))
  # group by collision function, as mjx does, keeping geom order inside a group
  pairs.sort(key=lambda p: p[0])
  c_kind, c_sub, c_g1, c_g2 = [], [], [], []
  for kind, a, b in pairs:
    for s in range(S.CON_SLOTS[kind]):
      c_kind.append(kind)
      c_sub.append(s)
      c_g1.append(a)
      c_g2.append(b)
  c_g1 = np.array(c_g1, dtype=np.int64)
  c_g2 = np.array(c_g2, dtype=np.int64)
  ncon = c_g1.shape[0]
  fr5 = lambda f: np.array([f[0], f[0], f[1], f[2], f[2]])
  contacts = S.ContactSlots(
      kind=np.array(c_kind, dtype=np.int64), sub=np.array(c_sub, dtype=np.int64),
      geom1=c_g1, geom2=c_g2,
      link_a=g_body[c_g1] - 1 if ncon else np.zeros(0, np.int64),
      link_b=g_body[c_g2] - 1 if ncon else np.zeros(0, np.int64),
      friction=np.array([np.maximum(fr5(g_fric[a]), fr5(g_fric[b]))
                         for a, b in zip(c_g1, c_g2)]).reshape(ncon, 5),
      solref=np.array([0.5 * (g_sr[a] + g_sr[b]) for a, b in zip(c_g1, c_g2)]).reshape(ncon, 2),
      solimp=np.array([0.5 * (g_si[a] + g_si[b]) for a, b in zip(c_g1, c_g2)]).reshape(ncon, 5),
      elasticity=np.array([0.5 * (elasticity[a] + elasticity[b])
                           for a, b in zip(c_g1, c_g2)]).reshape(ncon))

  dof = S.DoF(
      motion=S.Motion(ang=dof_ang, vel=dof_vel),
      armature=np.array(armature), stiffness=np.array(stiffness),
      damping=np.array(damping),
      limit=(np.array(lo), np.array(hi)) if any_limited else None,
      invweight=np.zeros(nv), solver_params=np.array(solp).reshape(nv, 7))
  link = S.Link(
      transform=S.Transform(pos=link_pos, rot=link_rot),
      joint=S.Transform(pos=joint_pos, rot=np.tile([1.0, 0, 0, 0], (nl, 1))),
      inertia=S.Inertia(transform=S.Transform(pos=ipos, rot=iquat), i=inertia_i,
                        mass=mass),
      invweight=np.zeros(nl))
  q0 = np.array(q0)
  init_q = np.atleast_1d(custom['init_qpos']).astype(np.float64) if 'init_qpos' in custom else q0
  sys = S.System(
      gravity=gravity, dt=dt, link=link, dof=dof, actuator=actuator,
      init_q=init_q, link_types=link_types, link_parents=link_parents,
      link_names=[b.name for b in bodies[1:]],
      matrix_inv_iterations=int(custom['matrix_inv_iterations']),
      solver_iterations=iterations, solver_maxls=int(custom['solver_maxls']),
      geom_type=g_type, geom_bodyid=g_body, geom_pos=g_pos, geom_quat=g_quat,
      geom_size=g_size, geom_friction=g_fric, geom_solref=g_sr, geom_solimp=g_si,
      geom_contype=g_ct, geom_conaffinity=g_ca, elasticity=elasticity,
      contacts=contacts, viscosity=viscosity, density=density,
      name=name or root.attrib.get('model', ''),
      geom_rgba=np.array(g_rgba, dtype=np.float64).reshape(ngeom, 4))
  _set_invweights(sys, q0)
  return sys


def load(path: str) -> S.System:
  with open(path) as f:
    return loads(f.read(), name=os.path.splitext(os.path.basename(path))[0])


def load_asset(name: str) -> S.System:
  """Loads one of the packaged workload models by file stem."""
  return load(os.path.join(_ASSET_DIR, name + '.xml'))


# --------------------------------------------------------------------------
# invweight0 at qpos0
# --------------------------------------------------------------------------


def _set_invweights(sys: S.System, q0: np.ndarray):
  """Fills link.invweight / dof.invweight like MuJoCo's body_/dof_invweight0."""
  nl, nv = sys.num_links(), sys.qd_size()
  if nv == 0:
    return
  qr, dr = sys.q_ranges(), sys.dof_ranges()
  xpos, xrot = np.zeros((nl, 3)), np.zeros((nl, 4))
  # world frames at q0, with the joint anchor convention of brax/kinematics.py
  anchor_w = np.zeros((nl, 3))
  for i, t in enumerate(sys.link_types):
    p = sys.link_parents[i]
    ppos, prot = (xpos[p], xrot[p]) if p >= 0 else (np.zeros(3), np.array([1.0, 0, 0, 0]))
    if t == 'f':
      jpos, jrot = q0[qr[i][0]:qr[i][0] + 3], q0[qr[i][0] + 3:qr[i][0] + 7]
    else:
      jpos, jrot = np.zeros(3), np.array([1.0, 0, 0, 0])
    lpos = sys.link.transform.pos[i] + _qrot(jpos, sys.link.transform.rot[i])
    lrot = _qmul(sys.link.transform.rot[i], jrot)
    xpos[i] = ppos + _qrot(lpos, prot)
    xrot[i] = _qmul(prot, lrot)
    anchor_w[i] = xpos[i] + _qrot(sys.link.joint.pos[i], xrot[i])
  com = np.array([xpos[i] + _qrot(sys.link.inertia.transform.pos[i], xrot[i])
                  for i in range(nl)]).reshape(nl, 3)
  iw = []
  for i in range(nl):
    r = _qmat(xrot[i]) @ _qmat(sys.link.inertia.transform.rot[i])
    iw.append(r @ sys.link.inertia.i[i] @ r.T)
  # dof axes in world
  ancestors = []
  for i in range(nl):
    a, j = [], i
    while j >= 0:
      a.append(j)
      j = sys.link_parents[j]
    ancestors.append(set(a))

  def jac(i, point):
    jp_, jr_ = np.zeros((3, nv)), np.zeros((3, nv))
    for l in ancestors[i]:
      rot = xrot[l]
      for k, d in enumerate(dr[l]):
        if sys.link_types[l] == 'f':
          if k < 3:
            jp_[k, d] = 1.0
          else:
            ax = _qrot(np.eye(3)[k - 3], rot)
            jr_[:, d] = ax
            jp_[:, d] = np.cross(ax, point - anchor_w[l])
        else:
          ang = _qrot(sys.dof.motion.ang[d], rot)
          vel = _qrot(sys.dof.motion.vel[d], rot)
          jr_[:, d] = ang
          jp_[:, d] = vel + np.cross(ang, point - anchor_w[l])
    return jp_, jr_

  m = np.diag(sys.dof.armature.astype(np.float64))
  jacs = []
  for i in range(nl):
    jp_, jr_ = jac(i, com[i])
    jacs.append((jp_, jr_))
    m += sys.link.inertia.mass[i] * jp_.T @ jp_ + jr_.T @ iw[i] @ jr_
  minv = np.linalg.inv(m)
  for i in range(nl):
    j6 = np.concatenate(jacs[i])
    a = j6 @ minv @ j6.T
    sys.link.invweight[i] = np.trace(a[:3, :3]) / 3.0
  diag = np.diag(minv).copy()
  for i, t in enumerate(sys.link_types):
    d = dr[i]
    if t == 'f':
      diag[d[0]:d[0] + 3] = diag[d[0]:d[0] + 3].mean()
      diag[d[3]:d[3] + 3] = diag[d[3]:d[3] + 3].mean()
  sys.dof.invweight[:] = diag
