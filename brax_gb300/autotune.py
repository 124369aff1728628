"""Launch-shape autotuner: lanes per env and envs per CTA for each nv bucket.

For every nv bucket present in a batch (nv <= 8, 16, 32, 64) the tuner builds
a batch of that bucket's models alone (with their env counts), times a short
rollout of it for every candidate shape with CUDA events, and keeps the
fastest.  Results are cached in a JSON file keyed by the GPU name, the bucket
and the bucket's models and env counts, so a later process with the same batch
reads them instead of timing again.  The cache lives next to the built library
(``brax_gb300/_lib/autotune.json``) unless ``BRAXG_TUNE_CACHE`` names another
file.
"""

from __future__ import annotations

import hashlib
import json
import os
import threading
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from brax_gb300 import _native as N
from brax_gb300 import model_pack
from brax_gb300 import pipeline as P

BUCKETS = (8, 16, 32, 64)
# per-CTA shared memory of the tuned launch: one CTA per SM (all of an SM's
# warps then run the same stage's code), as the batch default; shapes are
# timed under the same limit as the combined launch that uses them
SMEM_PER_CTA = 227 * 1024 - 16
_lock = threading.Lock()


def cache_path() -> str:
  return os.environ.get('BRAXG_TUNE_CACHE') or os.path.join(N.LIB_DIR, 'autotune.json')


def bucket_of(nv: int) -> int:
  for b in BUCKETS:
    if nv <= b:
      return b
  raise NotImplementedError(f'nv {nv} is above the largest bucket {BUCKETS[-1]}')


def candidates(bucket: int) -> List[Tuple[int, int]]:
  """(threads_per_env, envs_per_cta) pairs; envs_per_cta 0 = as many as the
  CTA's shared memory and 512 threads hold."""
  out = []
  lanes = (16, 32) if bucket <= 32 else (32,)
  for t in lanes:
    for e in (0, 4, 8, 12, 16) if t == 32 else (0, 8, 16, 24, 32):
      out.append((t, e))
  return out


def _key(device: torch.device, bucket: int, systems, n_env, n_frames) -> str:
  h = hashlib.sha1()
  for s, n, f in zip(systems, n_env, n_frames):
    h.update(model_pack.pack(s).tobytes())
    h.update(np.asarray([n, f], np.int64).tobytes())
  name = torch.cuda.get_device_name(device)
  return f'{name}|nv<={bucket}|{h.hexdigest()[:16]}'


def _load() -> Dict:
  try:
    with open(cache_path()) as f:
      return json.load(f)
  except (OSError, ValueError):
    return {}


def _store(table: Dict):
  path = cache_path()
  os.makedirs(os.path.dirname(path), exist_ok=True)
  tmp = path + f'.{os.getpid()}.tmp'
  with open(tmp, 'w') as f:
    json.dump(table, f, indent=1, sort_keys=True)
  os.replace(tmp, path)


def _time_shape(systems, n_env, n_frames, shape, device, n_steps: int, reps: int, smem: int) -> float:
  return _time_batch(systems, n_env, n_frames, [(BUCKETS[-1], shape[0], shape[1])], device, n_steps, reps,
                     smem)


def _time_batch(systems, n_env, n_frames, shapes, device, n_steps: int, reps: int, smem: int = 0) -> float:
  """Median CUDA-event time (ms) of an n_steps rollout of the batch."""
  from brax_gb300.batch import Batch
  from brax_gb300 import workloads as W
  b = Batch(systems, n_env, n_frames, shapes=shapes, smem_per_cta=smem, device=device)
  rng = np.random.default_rng(0)
  qs, qds, acts = [], [], []
  for s, n in zip(systems, n_env):
    q, qd = W.reset(s, n, rng)
    qs.append(q)
    qds.append(qd)
    acts.append(np.stack([W.actions(s, n, rng) for _ in range(n_steps)]))
  state = b.init(b.concat(qs, 'q'), b.concat(qds, 'qd'))
  act = b.concat_steps(acts, 'act') if b.totals['act'] else None
  out = b.alloc()
  b.rollout(state, act, n_steps, out=out)  # warm-up
  stream = torch.cuda.current_stream(device)
  times = []
  for _ in range(reps):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.rollout(state, act, n_steps, out=out)
    e1.record(stream)
    e1.synchronize()
    times.append(e0.elapsed_time(e1))
  return float(np.median(times))


def tune_batch(systems: Sequence, n_env: Sequence[int], n_frames: Optional[Sequence[int]] = None,
               device=None, n_steps: int = 8, reps: int = 5, use_cache: bool = True,
               verbose: bool = False) -> List[Tuple[int, int, int]]:
  """Shapes [(nv_max, threads_per_env, envs_per_cta)] for ``Batch(shapes=...)``,
  one per nv bucket present, each the fastest candidate for that bucket's
  models timed alone; the combination is then timed on the whole batch
  against the default shape (32 lanes, envs per CTA filling the CTA) and the
  faster of the two is returned (an empty list for the default)."""
  device = torch.device('cuda') if device is None else torch.device(device)
  if device.index is None:
    device = torch.device('cuda', torch.cuda.current_device())
  n_frames = [1] * len(systems) if n_frames is None else list(n_frames)
  groups: Dict[int, List[int]] = {}
  for g, s in enumerate(systems):
    if n_env[g] > 0:
      groups.setdefault(bucket_of(s.qd_size()), []).append(g)
  with _lock:
    table = _load() if use_cache else {}
  shapes = []
  dirty = False
  for bucket in sorted(groups):
    idx = groups[bucket]
    sys_b = [systems[g] for g in idx]
    ne_b = [n_env[g] for g in idx]
    nf_b = [n_frames[g] for g in idx]
    key = _key(device, bucket, sys_b, ne_b, nf_b)
    hit = table.get(key)
    if hit is None:
      results = {}
      for shape in candidates(bucket):
        try:
          results[shape] = _time_shape(sys_b, ne_b, nf_b, shape, device, n_steps, reps, SMEM_PER_CTA)
        except (ValueError, NotImplementedError):
          continue  # shape does not fit this bucket's models
        if verbose:
          print(f'nv<={bucket} threads {shape[0]} envs/cta {shape[1]}: {results[shape]:.3f} ms')
      if not results:
        raise NotImplementedError(f'no launch shape fits the nv<={bucket} models')
      best = min(results, key=results.get)
      hit = {'threads_per_env': best[0], 'envs_per_cta': best[1], 'ms': results[best],
             'timed': {f'{t}x{e}': ms for (t, e), ms in results.items()}}
      table[key] = hit
      dirty = True
    shapes.append((bucket, hit['threads_per_env'], hit['envs_per_cta']))
  if len(groups) > 0:  # the combination against the default on the whole batch
    all_idx = [g for idx in groups.values() for g in idx]
    key = _key(device, 0, [systems[g] for g in all_idx], [n_env[g] for g in all_idx],
               [n_frames[g] for g in all_idx]) + '|' + repr(shapes)
    hit = table.get(key)
    if hit is None:
      live = [g for g in range(len(systems)) if n_env[g] > 0]
      args = ([systems[g] for g in live], [n_env[g] for g in live], [n_frames[g] for g in live])
      tuned = _time_batch(*args, shapes, device, 4 * n_steps, reps)
      default = _time_batch(*args, [], device, 4 * n_steps, reps)
      hit = {'use_tuned': tuned <= default, 'tuned_ms': tuned, 'default_ms': default}
      table[key] = hit
      dirty = True
      if verbose:
        print(f'whole batch: tuned {tuned:.3f} ms, default {default:.3f} ms')
    if not hit['use_tuned']:
      shapes = []
  if dirty and use_cache:
    with _lock:
      merged = _load()
      merged.update(table)
      _store(merged)
  return shapes
