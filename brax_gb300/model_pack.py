"""Packs a ``System`` into the 32-bit word descriptor the kernels consume.

The word layout is declared once, in ``csrc/model_layout.h``; this module reads
the enum from that header so the two sides cannot drift apart.
"""

from __future__ import annotations

import os
import re
from typing import Dict

import numpy as np

from brax_gb300 import system as S

_HDR = os.path.join(os.path.dirname(__file__), 'csrc', 'model_layout.h')


def _read_enum() -> Dict[str, int]:
  text = open(_HDR).read()
  body = text[text.index('enum BxmHeader'):]
  body = body[body.index('{') + 1: body.index('};')]
  out, k = {}, 0
  for line in body.splitlines():
    line = line.split('//')[0].strip().rstrip(',')
    if not line:
      continue
    m = re.match(r'(\w+)\s*(=\s*(\d+))?$', line)
    if not m:
      raise ValueError(f'cannot parse model_layout.h line: {line}')
    if m.group(3) is not None:
      k = int(m.group(3))
    out[m.group(1)] = k
    k += 1
  return out


H = _read_enum()
MAGIC = 0x42584D31
VERSION = 1
TYPE_CODE = {'f': 0, '1': 1, '2': 2, '3': 3}


def pack(sys: S.System) -> np.ndarray:
  """Returns the descriptor as an int32 array (floats stored as bit patterns)."""
  nl, nq, nv, nu = sys.num_links(), sys.q_size(), sys.qd_size(), sys.act_size()
  cs = sys.contacts
  ncon = cs.n
  nlim = sys.n_limit_rows()
  depth = sys.link_depth()
  nlevel = (max(depth) + 1) if nl else 0
  levels = [[i for i in range(nl) if depth[i] == d] for d in range(nlevel)]
  qadr, dadr = [], []
  qa = da = 0
  for t in sys.link_types:
    qadr.append(qa)
    dadr.append(da)
    qa += S.Q_WIDTHS[t]
    da += S.QD_WIDTHS[t]
  children = [[c for c in range(nl) if sys.link_parents[c] == i] for i in range(nl)]
  child_start = np.cumsum([0] + [len(c) for c in children])
  roots = sys.link_root()
  dof_link = sys.dof_link()
  if nv > 64:
    raise NotImplementedError('models with more than 64 dofs are not supported')
  anc = np.zeros((nl, 2), np.uint32)
  for i in range(nl):
    mask, j = 0, i
    while j >= 0:
      for d in range(dadr[j], dadr[j] + S.QD_WIDTHS[sys.link_types[j]]):
        mask |= 1 << d
      j = sys.link_parents[j]
    anc[i, 0] = mask & 0xFFFFFFFF
    anc[i, 1] = (mask >> 32) & 0xFFFFFFFF
  lim_dof = sys.qd_idx('123') if nlim else np.zeros(0, np.int64)
  lim_q = sys.q_idx('123') if nlim else np.zeros(0, np.int64)
  mass = sys.link.inertia.mass
  root_mass = np.array([sum(mass[j] for j in range(nl) if roots[j] == roots[i])
                        for i in range(nl)])
  inv = sys.link.invweight
  con_invw = np.array([(inv[a] if a > -1 else 0.0) + inv[b]
                       for a, b in zip(cs.link_a, cs.link_b)])
  g1, g2 = cs.geom1, cs.geom2

  ints = {
      'BXM_O_LINK_PARENT': np.array(sys.link_parents),
      'BXM_O_LINK_TYPE': np.array([TYPE_CODE[t] for t in sys.link_types]),
      'BXM_O_LINK_QADR': np.array(qadr), 'BXM_O_LINK_DADR': np.array(dadr),
      'BXM_O_LINK_ROOT': np.array(roots),
      'BXM_O_LEVEL_START': np.cumsum([0] + [len(l) for l in levels]),
      'BXM_O_LEVEL_LINKS': np.array(sum(levels, [])),
      'BXM_O_CHILD_START': child_start,
      'BXM_O_CHILD_IDX': np.array(sum(children, [])),
      'BXM_O_DOF_LINK': dof_link,
      'BXM_O_LINK_ANC': anc.reshape(-1).view(np.int32),
      'BXM_O_LIM_DOF': lim_dof, 'BXM_O_LIM_QADR': lim_q,
      'BXM_O_ACT_QID': sys.actuator.q_id, 'BXM_O_ACT_QDID': sys.actuator.qd_id,
      'BXM_O_CON_KIND': cs.kind, 'BXM_O_CON_SUB': cs.sub,
      'BXM_O_CON_LA': cs.link_a, 'BXM_O_CON_LB': cs.link_b,
  }
  lo = sys.dof.limit[0][lim_dof] if nlim else np.zeros(0)
  hi = sys.dof.limit[1][lim_dof] if nlim else np.zeros(0)
  floats = {
      'BXM_O_LT_POS': sys.link.transform.pos, 'BXM_O_LT_ROT': sys.link.transform.rot,
      'BXM_O_LJ_POS': sys.link.joint.pos,
      'BXM_O_LI_POS': sys.link.inertia.transform.pos,
      'BXM_O_LI_ROT': sys.link.inertia.transform.rot,
      'BXM_O_LI_I': sys.link.inertia.i, 'BXM_O_LI_MASS': mass,
      'BXM_O_L_INVW': inv, 'BXM_O_ROOT_MASS': root_mass,
      'BXM_O_D_ANG': sys.dof.motion.ang, 'BXM_O_D_VEL': sys.dof.motion.vel,
      'BXM_O_D_ARM': sys.dof.armature, 'BXM_O_D_STIFF': sys.dof.stiffness,
      'BXM_O_D_DAMP': sys.dof.damping, 'BXM_O_D_INVW': sys.dof.invweight,
      'BXM_O_LIM_LO': lo, 'BXM_O_LIM_HI': hi,
      'BXM_O_LIM_INVW': sys.dof.invweight[lim_dof] if nlim else np.zeros(0),
      'BXM_O_LIM_SOLP': sys.dof.solver_params[lim_dof] if nlim else np.zeros((0, 7)),
      'BXM_O_ACT_CR': sys.actuator.ctrl_range, 'BXM_O_ACT_FR': sys.actuator.force_range,
      'BXM_O_ACT_GAIN': sys.actuator.gain, 'BXM_O_ACT_GEAR': sys.actuator.gear,
      'BXM_O_ACT_BQ': sys.actuator.bias_q, 'BXM_O_ACT_BQD': sys.actuator.bias_qd,
      'BXM_O_CON_G1POS': sys.geom_pos[g1], 'BXM_O_CON_G1QUAT': sys.geom_quat[g1],
      'BXM_O_CON_G1SIZE': sys.geom_size[g1],
      'BXM_O_CON_G2POS': sys.geom_pos[g2], 'BXM_O_CON_G2QUAT': sys.geom_quat[g2],
      'BXM_O_CON_G2SIZE': sys.geom_size[g2],
      'BXM_O_CON_FRIC': cs.friction[:, 0] if ncon else np.zeros(0),
      'BXM_O_CON_INVW': con_invw,
      'BXM_O_CON_SOLP': (np.concatenate([cs.solref, cs.solimp], axis=1)
                         if ncon else np.zeros((0, 7))),
      'BXM_O_LI_BOX': fluid_box(sys),
  }
  words = [np.zeros(H['BXM_HEADER_WORDS'], np.int32)]
  off = H['BXM_HEADER_WORDS']
  hdr = words[0]

  def put(name, arr):
    nonlocal off
    arr = np.ascontiguousarray(arr).reshape(-1)
    hdr[H[name]] = off
    # keep every array 4-word aligned (16-byte vector loads)
    n = (arr.shape[0] + 3) // 4 * 4
    buf = np.zeros(n, np.int32)
    buf[:arr.shape[0]] = arr
    words.append(buf)
    off += n

  for k, v in ints.items():
    put(k, np.asarray(v, np.int64).astype(np.int32) if v.dtype != np.int32 else v)
  for k, v in floats.items():
    put(k, np.asarray(v, np.float64).astype(np.float32).view(np.int32))
  f32 = lambda x: np.array([x], np.float32).view(np.int32)[0]
  hdr[H['BXM_H_MAGIC']] = np.int64(MAGIC).astype(np.int32)
  hdr[H['BXM_H_VERSION']] = VERSION
  hdr[H['BXM_H_WORDS']] = off
  for k, v in (('NL', nl), ('NQ', nq), ('NV', nv), ('NU', nu), ('NCON', ncon),
               ('NLIM', nlim), ('M', 4 * ncon + nlim), ('NLEVEL', nlevel),
               ('NS_ITERS', sys.matrix_inv_iterations),
               ('PG_ITERS', sys.solver_iterations), ('PG_MAXLS', sys.solver_maxls),
               ('NROOT', len(set(roots)))):
    hdr[H['BXM_H_' + k]] = v
  hdr[H['BXM_H_DT']] = f32(sys.dt)
  hdr[H['BXM_H_GX']], hdr[H['BXM_H_GY']], hdr[H['BXM_H_GZ']] = (f32(g) for g in sys.gravity)
  hdr[H['BXM_H_PG_TOL']] = f32(1e-3)
  hdr[H['BXM_H_FLUID']] = int(sys.enable_fluid)
  hdr[H['BXM_H_VISC']] = f32(sys.viscosity)
  hdr[H['BXM_H_DENS']] = f32(sys.density)
  return np.concatenate(words)


def fluid_box(sys: S.System) -> np.ndarray:
  """[nl, 3] edge lengths of the box with each link's mass and principal
  moments (brax/fluid.py:71-76): sqrt(6 (tr(I) - 2 I_kk) / m), floored at
  1e-12 before the square root."""
  i = np.asarray(sys.link.inertia.i, np.float64).reshape(-1, 3, 3)
  d = np.diagonal(i, axis1=-2, axis2=-1)
  v = 6.0 * np.maximum(d.sum(-1, keepdims=True) - 2.0 * d, 1e-12)
  return np.sqrt(v / np.asarray(sys.link.inertia.mass, np.float64)[:, None])
