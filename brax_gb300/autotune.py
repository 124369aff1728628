"""Launch-shape autotuner: lanes per env and envs per CTA for each nv bucket.

For the nv buckets present in a batch (nv <= 8, 16, 32, 64) the tuner runs a
coordinate descent on the whole batch: each bucket's candidate shapes are
timed (CUDA events, a short rollout of the whole batch, every model's work
items interleaved in one launch as they run) with the other buckets at their
current shapes, and a candidate is kept only if it beats the current shapes.
Results are cached in a JSON file keyed by the GPU name and the batch's
models, env counts and frames, so a later process with the same batch reads
them instead of timing again.  The cache lives next to the built library
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


def default_shape(bucket: int) -> Tuple[int, int, int]:
  """The shape a model of this bucket gets without tuning (braxg_batch_create:
  16 lanes per env for nv <= 8, else 32; envs per CTA filling the CTA)."""
  return (bucket, 16 if bucket <= 8 else 32, 0)


def tune_batch(systems: Sequence, n_env: Sequence[int], n_frames: Optional[Sequence[int]] = None,
               device=None, n_steps: int = 16, reps: int = 5, use_cache: bool = True,
               verbose: bool = False, min_gain: float = 0.01) -> List[Tuple[int, int, int]]:
  """Shapes [(nv_max, threads_per_env, envs_per_cta)] for ``Batch(shapes=...)``
  by coordinate descent on the whole batch: starting from the default shape
  of every nv bucket present, each bucket in turn tries its candidates with
  the other buckets at their current shapes, timing an n_steps rollout of the
  whole batch (the models of all buckets interleaved in one launch, as they
  run), and keeps a candidate only if it is at least ``min_gain`` faster than
  the current shapes.  Returns [] when the default shapes are kept."""
  device = torch.device('cuda') if device is None else torch.device(device)
  if device.index is None:
    device = torch.device('cuda', torch.cuda.current_device())
  n_frames = [1] * len(systems) if n_frames is None else list(n_frames)
  live = [g for g in range(len(systems)) if n_env[g] > 0]
  if not live:
    return []
  args = ([systems[g] for g in live], [n_env[g] for g in live], [n_frames[g] for g in live])
  buckets = sorted({bucket_of(systems[g].qd_size()) for g in live})
  key = _key(device, 0, *args) + '|descent'
  with _lock:
    table = _load() if use_cache else {}
  hit = table.get(key)
  if hit is None:
    cur = {b: default_shape(b) for b in buckets}
    shape_list = lambda c: [c[b] for b in buckets]
    best = default_ms = _time_batch(*args, shape_list(cur), device, n_steps, reps)
    timed = {'default': default_ms}
    for b in buckets:
      for t, e in candidates(b):
        trial = dict(cur)
        trial[b] = (b, t, e)
        if trial == cur:
          continue
        try:
          ms = _time_batch(*args, shape_list(trial), device, n_steps, reps)
        except (ValueError, NotImplementedError):
          continue  # the shape does not fit this bucket's models
        timed[f'nv<={b} {t}x{e}'] = ms
        if verbose:
          print(f'nv<={b} threads {t} envs/cta {e}: {ms:.3f} ms (current best {best:.3f})')
        if ms < best * (1.0 - min_gain):
          cur, best = trial, ms
    shapes = [] if all(cur[b] == default_shape(b) for b in buckets) else shape_list(cur)
    hit = {'shapes': shapes, 'ms': best, 'default_ms': default_ms, 'timed': timed}
    table[key] = hit
    if use_cache:
      with _lock:
        merged = _load()
        merged[key] = hit
        _store(merged)
  return [tuple(s) for s in hit['shapes']]


def report(systems: Sequence, n_env: Sequence[int], n_frames: Optional[Sequence[int]] = None,
           device=None) -> Optional[Dict]:
  """What tune_batch measured for this batch (from the cache): the default
  shapes' time, the kept shapes' time and every candidate's, in ms of an
  n_steps rollout of the whole batch; None if it was never tuned."""
  device = torch.device('cuda') if device is None else torch.device(device)
  if device.index is None:
    device = torch.device('cuda', torch.cuda.current_device())
  n_frames = [1] * len(systems) if n_frames is None else list(n_frames)
  live = [g for g in range(len(systems)) if n_env[g] > 0]
  args = ([systems[g] for g in live], [n_env[g] for g in live], [n_frames[g] for g in live])
  with _lock:
    return _load().get(_key(device, 0, *args) + '|descent')
