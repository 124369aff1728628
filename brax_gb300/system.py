"""Model container for the generalized-coordinates physics step.

The field names and shapes follow brax's ``System`` (brax/base.py:415-540) and
the sub-structures ``Link``/``DoF``/``Actuator``/``Inertia``/``Transform``/
``Motion`` (brax/base.py:170-394), restricted to what the generalized pipeline
(brax/generalized/pipeline.py:32-94) reads.  Arrays are host numpy (float64
while the model is compiled; the device descriptor is float32).

One addition has no brax field of its own: ``contacts``, the static table of
candidate contact slots.  brax obtains it at trace time from
``mjx.make_data(sys)`` + ``mjx.collision`` (brax/contact.py:38,57); here the
model compiler (``brax_gb300.mjcf``) fixes it once per model.
"""

from __future__ import annotations

import dataclasses
from typing import List, Optional, Tuple

import numpy as np

# brax/base.py:33-34
Q_WIDTHS = {'f': 7, '1': 1, '2': 2, '3': 3}
QD_WIDTHS = {'f': 6, '1': 1, '2': 2, '3': 3}

# MuJoCo geom type numbering (mjtGeom), kept so that pair ordering matches.
GEOM_PLANE, GEOM_HFIELD, GEOM_SPHERE, GEOM_CAPSULE = 0, 1, 2, 3
GEOM_ELLIPSOID, GEOM_CYLINDER, GEOM_BOX, GEOM_MESH = 4, 5, 6, 7

# Collision kinds of one contact slot (one slot = one contact).  The pair
# (geom1, geom2) is ordered so that geom1 has the lower geom type, and the
# contact normal points from geom1 to geom2 (MuJoCo convention).
CON_PLANE_SPHERE = 0    # 1 contact per pair
CON_PLANE_CAPSULE = 1   # 2 contacts per pair (segment end +, end -)
CON_PLANE_BOX = 2       # 4 contacts per pair (mjx's plane-convex manifold of the box's vertices)
CON_SPHERE_SPHERE = 3   # 1 contact
CON_SPHERE_CAPSULE = 4  # 1 contact
CON_CAPSULE_CAPSULE = 5  # 1 contact
CON_SLOTS = {CON_PLANE_SPHERE: 1, CON_PLANE_CAPSULE: 2, CON_PLANE_BOX: 4,
             CON_SPHERE_SPHERE: 1, CON_SPHERE_CAPSULE: 1,
             CON_CAPSULE_CAPSULE: 1}
# (type1, type2) -> kind, for type1 <= type2
CON_KIND = {
    (GEOM_PLANE, GEOM_SPHERE): CON_PLANE_SPHERE,
    (GEOM_PLANE, GEOM_CAPSULE): CON_PLANE_CAPSULE,
    (GEOM_PLANE, GEOM_BOX): CON_PLANE_BOX,
    (GEOM_SPHERE, GEOM_SPHERE): CON_SPHERE_SPHERE,
    (GEOM_SPHERE, GEOM_CAPSULE): CON_SPHERE_CAPSULE,
    (GEOM_CAPSULE, GEOM_CAPSULE): CON_CAPSULE_CAPSULE,
}


@dataclasses.dataclass
class Transform:
  pos: np.ndarray  # (..., 3)
  rot: np.ndarray  # (..., 4) quaternion w, x, y, z


@dataclasses.dataclass
class Motion:
  ang: np.ndarray  # (..., 3)
  vel: np.ndarray  # (..., 3)


@dataclasses.dataclass
class Inertia:
  transform: Transform
  i: np.ndarray      # (..., 3, 3)
  mass: np.ndarray   # (...,)


@dataclasses.dataclass
class Link:
  transform: Transform  # link frame relative to parent link frame
  joint: Transform      # joint frame relative to link frame
  inertia: Inertia      # com frame, inertia and mass of the link
  invweight: np.ndarray  # translational inverse weight at init (body_invweight0)


@dataclasses.dataclass
class DoF:
  motion: Motion
  armature: np.ndarray
  stiffness: np.ndarray
  damping: np.ndarray
  limit: Optional[Tuple[np.ndarray, np.ndarray]]
  invweight: np.ndarray
  solver_params: np.ndarray  # (nv, 7): solref(2) + solimp(5)


@dataclasses.dataclass
class Actuator:
  q_id: np.ndarray
  qd_id: np.ndarray
  ctrl_range: np.ndarray   # (nu, 2)
  force_range: np.ndarray  # (nu, 2)
  gain: np.ndarray
  gear: np.ndarray
  bias_q: np.ndarray
  bias_qd: np.ndarray


@dataclasses.dataclass
class ContactSlots:
  """Static candidate contacts (one row per contact slot)."""
  kind: np.ndarray        # (ncon,) CON_* code
  sub: np.ndarray         # (ncon,) index of the contact within its pair
  geom1: np.ndarray       # (ncon,)
  geom2: np.ndarray       # (ncon,)
  link_a: np.ndarray      # (ncon,) geom_bodyid[geom1] - 1 (-1 = world)
  link_b: np.ndarray      # (ncon,) geom_bodyid[geom2] - 1
  friction: np.ndarray    # (ncon, 5) mixed friction (slide, slide, spin, roll, roll)
  solref: np.ndarray      # (ncon, 2) mixed solref
  solimp: np.ndarray      # (ncon, 5) mixed solimp
  elasticity: np.ndarray  # (ncon,)

  @property
  def n(self) -> int:
    return int(self.kind.shape[0])


@dataclasses.dataclass
class System:
  """A compiled model (the subset of brax.base.System the step reads)."""
  gravity: np.ndarray
  dt: float                      # sys.opt.timestep
  link: Link
  dof: DoF
  actuator: Actuator
  init_q: np.ndarray
  link_types: str
  link_parents: Tuple[int, ...]
  link_names: List[str]
  matrix_inv_iterations: int
  solver_iterations: int
  solver_maxls: int
  # geoms (MuJoCo geom_* fields)
  geom_type: np.ndarray
  geom_bodyid: np.ndarray
  geom_pos: np.ndarray
  geom_quat: np.ndarray
  geom_size: np.ndarray
  geom_friction: np.ndarray
  geom_solref: np.ndarray
  geom_solimp: np.ndarray
  geom_contype: np.ndarray
  geom_conaffinity: np.ndarray
  elasticity: np.ndarray
  contacts: ContactSlots
  viscosity: float = 0.0
  density: float = 0.0
  name: str = ''
  geom_rgba: Optional[np.ndarray] = None  # (ngeom, 4), MJCF rgba (default 0.5 0.5 0.5 1)

  @property
  def enable_fluid(self) -> bool:
    return bool(self.viscosity > 0 or self.density > 0)

  # --- brax/base.py:482-540 -------------------------------------------------
  def num_links(self) -> int:
    return len(self.link_types)

  def q_size(self) -> int:
    return sum(Q_WIDTHS[t] for t in self.link_types)

  def qd_size(self) -> int:
    return sum(QD_WIDTHS[t] for t in self.link_types)

  def act_size(self) -> int:
    return int(self.actuator.q_id.shape[0])

  def dof_link(self, depth: bool = False) -> np.ndarray:
    idxs = []
    for i, t in enumerate(self.link_types):
      idxs.extend([i] * QD_WIDTHS[t])
    if depth:
      d = self.link_depth()
      count, within = {}, []
      for i in range(self.num_links()):
        within.append(count.get(d[i], 0))
        count[d[i]] = within[-1] + 1
      idxs = [within[i] for i in idxs]
    return np.array(idxs, dtype=np.int64)

  def dof_ranges(self) -> List[List[int]]:
    beg, ranges = 0, []
    for t in self.link_types:
      ranges.append(list(range(beg, beg + QD_WIDTHS[t])))
      beg += QD_WIDTHS[t]
    return ranges

  def q_ranges(self) -> List[List[int]]:
    beg, ranges = 0, []
    for t in self.link_types:
      ranges.append(list(range(beg, beg + Q_WIDTHS[t])))
      beg += Q_WIDTHS[t]
    return ranges

  def q_idx(self, link_type: str) -> np.ndarray:
    idx, idxs = 0, []
    for typ in self.link_types:
      if typ in link_type:
        idxs.extend(range(idx, idx + Q_WIDTHS[typ]))
      idx += Q_WIDTHS[typ]
    return np.array(idxs, dtype=np.int64)

  def qd_idx(self, link_type: str) -> np.ndarray:
    idx, idxs = 0, []
    for typ in self.link_types:
      if typ in link_type:
        idxs.extend(range(idx, idx + QD_WIDTHS[typ]))
      idx += QD_WIDTHS[typ]
    return np.array(idxs, dtype=np.int64)

  # --- derived static structure ---------------------------------------------
  def link_depth(self) -> List[int]:
    """Depth of each link (roots are 0), as brax/scan.py:87 computes it."""
    p = self.link_parents
    out = []
    for i in range(self.num_links()):
      d, j = 0, i
      while p[j] >= 0:
        d, j = d + 1, p[j]
      out.append(d)
    return out

  def link_root(self) -> List[int]:
    p = self.link_parents
    out = []
    for i in range(self.num_links()):
      j = i
      while p[j] >= 0:
        j = p[j]
      out.append(j)
    return out

  def n_limit_rows(self) -> int:
    """Rows of jac_limit (brax/generalized/constraint.py:115-132)."""
    if self.dof.limit is None:
      return 0
    return int(self.qd_idx('123').shape[0])

  def n_constraint_rows(self) -> int:
    return 4 * self.contacts.n + self.n_limit_rows()


# --------------------------------------------------------------------------
# JSON round trip of a compiled System (exact: floats are written as the
# shortest repr that reads back to the same float64)
# --------------------------------------------------------------------------
_CLASSES = {c.__name__: c for c in (Transform, Motion, Inertia, Link, DoF, Actuator, ContactSlots, System)}


def _enc(v):
  if dataclasses.is_dataclass(v):
    return {'__class__': type(v).__name__,
            **{f.name: _enc(getattr(v, f.name)) for f in dataclasses.fields(v)}}
  if isinstance(v, np.ndarray):
    return {'__ndarray__': v.dtype.str, 'shape': list(v.shape), 'data': v.reshape(-1).tolist()}
  if isinstance(v, tuple):
    return {'__tuple__': [_enc(x) for x in v]}
  if isinstance(v, list):
    return [_enc(x) for x in v]
  if isinstance(v, np.generic):
    return v.item()
  return v


def _dec(v):
  if isinstance(v, dict):
    if '__ndarray__' in v:
      return np.array(v['data'], dtype=np.dtype(v['__ndarray__'])).reshape(v['shape'])
    if '__tuple__' in v:
      return tuple(_dec(x) for x in v['__tuple__'])
    cls = _CLASSES[v['__class__']]
    return cls(**{k: _dec(x) for k, x in v.items() if k != '__class__'})
  if isinstance(v, list):
    return [_dec(x) for x in v]
  return v


def to_json(sys: System) -> str:
  """The System as JSON text (every field, bit-exact on reading back)."""
  import json
  return json.dumps(_enc(sys))


def from_json(text: str) -> System:
  import json
  return _dec(json.loads(text))
