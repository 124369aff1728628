#!/usr/bin/env python
"""Env-steps/s of the generalized-coordinates step on GB300.

Workload (the headline configuration): the quadruped (free sphere torso, 4
legs x 2 hinged capsules, nq 15, nv 14, 8 motors of gear 150, 9 geoms vs the
ground plane), 4096 envs, one env step = 5 pipeline steps of 0.01 s with one
action per env step (brax/envs/base.py:128-137), actions ~ U(-1, 1), resets
as brax/envs/ant.py:209-213 (init_q + U(-0.1, 0.1), qd ~ 0.1 N(0, 1)).

value  : env-steps/s with state and actions resident in HBM; each timed step
         is one braxg_step launch (5 frames x 4096 envs) timed with CUDA
         events on the launching stream; the L2 is flushed (a 256 MB write)
         before every timed step, outside the events.
e2e    : the same metric through the C ABI (braxg_step via ctypes) with host
         buffers: per step the actions are copied from pinned host memory,
         the step runs, and the observation (q, qd) is copied back to pinned
         host memory and waited for; wall-clock time.
--impl reference: the CPU baseline (the numpy restatement of the reference
         path, see oracle/) on all host cores.
"""

from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'env-steps/s fwd & fwd+adjoint, 4096-env quadruped, 1 GB300, at 1e-5 rel err'
WORKLOAD = 'quadruped'
N_FRAMES = 5
# what each --inverse choice runs (the bench line names the algorithm)
INVERSE_NAMES = {'cholesky': 'exact (symmetric sweep inverse; Cholesky pivots)',
                 'newton_schulz': 'newton_schulz (the reference algorithm, K from the model)'}


def parse(argv=None):
  p = argparse.ArgumentParser()
  p.add_argument('--gpus', type=int, default=1)
  p.add_argument('--steps', type=int, default=200)
  p.add_argument('--warmup', type=int, default=10)
  p.add_argument('--impl', default='braxg', choices=['braxg', 'reference'])
  p.add_argument('--envs', type=int, default=4096)
  p.add_argument('--inverse', default='cholesky', choices=['newton_schulz', 'cholesky'])
  p.add_argument('--threads-per-env', type=int, default=0)
  p.add_argument('--envs-per-cta', type=int, default=0)
  p.add_argument('--no-state-cache', dest='state_cache', action='store_false',
                 help='states carry no position-term cache (every step recomputes them)')
  p.add_argument('--cpu-sample-envs', type=int, default=256)
  p.add_argument('--no-cpu-baseline', action='store_true')
  p.add_argument('--no-adjoint', action='store_true')
  p.add_argument('--no-uneven', action='store_true')
  p.add_argument('--no-humanoid', action='store_true')
  p.add_argument('--adjoint-horizon', type=int, default=128,
                 help='env steps of the gradient workload (128 as configured; smaller for a profiler capture)')
  return p.parse_args(argv)


# ---------------------------------------------------------------------------
# algorithmic work per pipeline step (FLOPs and bytes), fixed formulas
# ---------------------------------------------------------------------------


def algorithmic(sys_, n_mv: float, carried_minv: bool = True):
  nl, nv, nq, nu = sys_.num_links(), sys_.qd_size(), sys_.q_size(), sys_.act_size()
  ncon = sys_.contacts.n
  m = sys_.n_constraint_rows()
  f_tree = 400 * nl + 150 * nv
  f_m = 11 * nv * nv + 33 * nv
  f_fact = nv ** 3 / 3 + m * nv * nv
  f_a = m * m * nv + 2 * m * nv + 100 * nv * ncon
  f_pg = 2 * m * m * n_mv
  f_tail = 2 * m * nv + 4 * nv * nv
  flops = f_tree + f_m + f_fact + f_a + f_pg + f_tail
  # state in/out + actions + link outputs, plus mass_mx_inv written (and read
  # back when it is carried, Newton-Schulz mode)
  bytes_env_step = 4 * (nq + nv + nu) + 4 * (nq + nv + 13 * nl) + (2 if carried_minv else 1) * 4 * nv * nv
  return flops, bytes_env_step


def profiled_traffic(kernel: str):
  """DRAM bytes (read + write) per launch of `kernel` on this workload, from the
  committed ncu summary profiles/<kernel>_quadruped_4096.md (a line
  `traffic_bytes_per_launch: N`); None when no summary is present."""
  path = os.path.join(ROOT, 'profiles', f'{kernel}_quadruped_4096.md')
  try:
    with open(path) as f:
      for line in f:
        if line.strip().startswith('traffic_bytes_per_launch:'):
          return int(float(line.split(':', 1)[1]))
  except OSError:
    pass
  return None


STATUS_BITS = {1: 'nonfinite', 2: 'not_spd', 4: 'no_gradient', 8: 'skipped', 16: 'bounds'}


def status_bits(status):
  """Envs per braxg_env_flags bit of a status array (bits that no env set are left out)."""
  import numpy as np
  st = np.asarray(status)
  return {name: int(((st & bit) != 0).sum()) for bit, name in STATUS_BITS.items() if ((st & bit) != 0).any()}


def max_over_ranks(seconds: float, device) -> float:
  """The slowest rank's time (one all-reduce MAX); the value itself on one rank."""
  import torch
  import torch.distributed as dist
  if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
    return seconds
  t = torch.tensor([seconds], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def whole_job_rate(units_per_rank: int, world: int, seconds: float) -> float:
  """Units all ranks processed (each rank a replica of the same size) over the
  slowest rank's time."""
  return units_per_rank * world / seconds


def WORKLOAD_SYS():
  from brax_gb300 import mjcf
  return mjcf.load_asset(WORKLOAD)


def workload_config(n: int, world: int):
  return {'workload': f'{WORKLOAD} nq 15 nv 14 nu 8, 9 geoms vs plane (17 contact slots), '
                      f'{n} envs per GPU, env step = {N_FRAMES} x 0.01 s',
          'envs_per_gpu': n, 'n_frames': N_FRAMES, 'parallelism': f'replicas x{world}'}


def load_nmv():
  path = os.path.join(ROOT, 'tests', 'golden', 'pg_matvecs.json')
  with open(path) as f:
    return json.load(f)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------


class ClockSampler:
  Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
       'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
       'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

  def __init__(self, index: int):
    self.index = index
    self.proc = None
    self.lines = []

  def __enter__(self):
    try:
      self.proc = subprocess.Popen(
          ['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.Q}',
           '--format=csv,noheader,nounits', '-lms', '50'],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
      self.t = threading.Thread(target=self._read, daemon=True)
      self.t.start()
      # the timed region starts once the sampler is producing samples
      deadline = time.perf_counter() + 5.0
      while not self.lines and time.perf_counter() < deadline and self.proc.poll() is None:
        time.sleep(0.01)
    except (OSError, FileNotFoundError):
      self.proc = None
    self.first = len(self.lines)
    return self

  def _read(self):
    for line in self.proc.stdout:
      self.lines.append(line.strip())

  def __exit__(self, *a):
    if self.proc is not None:
      self.proc.terminate()
      try:
        self.proc.wait(timeout=5)
      except subprocess.TimeoutExpired:
        self.proc.kill()
      self.t.join(timeout=2)

  def summary(self):
    sm, mx, reasons = [], None, set()
    names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
    # samples taken during the timed region (the last earlier one if none)
    lines = self.lines[self.first:] or self.lines[-1:]
    for line in lines:
      f = [x.strip() for x in line.split(',')]
      if len(f) < 9:
        continue
      try:
        sm.append(float(f[1]))
        mx = float(f[2])
      except ValueError:
        continue
      for k, nm in enumerate(names):
        if f[5 + k].lower().startswith('active'):
          reasons.add(nm)
    if not sm:
      return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled'], 'samples': 0}
    return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': mx, 'reasons': sorted(reasons),
            'samples': len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement (numpy, FP32) on all host cores
# ---------------------------------------------------------------------------


_CPU = {}


def _cpu_init(name, n, seed_base):
  """Pool initialiser: one oracle and one batch of envs per worker process."""
  from brax_gb300 import mjcf
  from oracle.pipeline import Oracle
  sys_ = mjcf.load_asset(name)
  o = Oracle(sys_, np.float32)
  rng = np.random.default_rng(seed_base + os.getpid())
  q = (sys_.init_q + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))).astype(np.float32)
  qd = (0.1 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32)
  _CPU.update(sys=sys_, o=o, rng=rng, s=o.init(q, qd), n=n)


def _cpu_run(args):
  """`warmup` untimed then `steps` timed env steps (N_FRAMES pipeline steps
  each) of this worker's envs; returns the timed steps' durations."""
  warmup, steps = args
  c = _CPU
  out = []
  for k in range(warmup + steps):
    t0 = time.perf_counter()
    act = c['rng'].uniform(-1, 1, (c['n'], c['sys'].act_size())).astype(np.float32)
    c['s'] = c['o'].env_step(c['s'], act, N_FRAMES)
    if k >= warmup:
      out.append(time.perf_counter() - t0)
  return out


class CpuReference:
  """The numpy FP32 restatement of the reference path (oracle/) on every
  host core: one spawn-started worker process per core (one BLAS thread
  each), each stepping its own batch of `sample_envs` envs through the same
  number of env steps, all at once.  A step is one env step of every
  worker's batch; the run's time is the slowest worker's."""

  def __init__(self, sample_envs: int):
    self.cores = os.cpu_count() or 1
    self.sample_envs = sample_envs
    keys = ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS')
    old = {k: os.environ.get(k) for k in keys}
    os.environ.update({k: '1' for k in keys})  # inherited by the workers
    try:
      self.pool = mp.get_context('spawn').Pool(self.cores, _cpu_init, (WORKLOAD, sample_envs, 100))
    finally:
      for k, v in old.items():
        if v is None:
          os.environ.pop(k, None)
        else:
          os.environ[k] = v

  def run(self, steps: int, warmup: int):
    """Returns (env-steps/s, per-step times of the slowest worker)."""
    res = self.pool.map(_cpu_run, [(warmup, steps)] * self.cores, chunksize=1)
    slowest = max(res, key=sum)
    return self.cores * self.sample_envs * steps / sum(slowest), slowest

  def describe(self, steps: int, wall) -> str:
    return (f'{self.cores} processes x {self.sample_envs} envs, {steps} timed env steps '
            f'({N_FRAMES} frames each) in each process at once, numpy FP32 restatement of the '
            f'reference path; slowest process {sum(wall):.1f} s, about '
            f'{self.cores * sum(wall):.0f} core-seconds')

  def close(self):
    self.pool.terminate()
    self.pool.join()


def cpu_baseline(sample_envs: int, steps: int = 8, warmup: int = 6):
  """Bounded sample of the reference path on the host cores: after 6 warm-up
  env steps (0.3 s, the quadrupeds have landed), 8 timed env steps."""
  ref = CpuReference(sample_envs)
  try:
    value, wall = ref.run(steps, warmup)
  finally:
    ref.close()
  return {'value': value, 'unit': 'env-steps/s', 'cores': ref.cores, 'kind': 'port',
          'sample': ref.describe(steps, wall)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------


def run_braxg(args):
  import torch
  import torch.distributed as dist
  world = int(os.environ.get('WORLD_SIZE', '1'))
  rank = int(os.environ.get('RANK', '0'))
  local = int(os.environ.get('LOCAL_RANK', '0'))
  torch.cuda.set_device(local)
  if world > 1:
    dist.init_process_group('nccl', device_id=torch.device('cuda', local))
  dev = torch.device('cuda', local)
  from brax_gb300 import _native, mjcf, pipeline
  sys_ = mjcf.load_asset(WORKLOAD)
  n = args.envs
  mode = pipeline.NEWTON_SCHULZ if args.inverse == 'newton_schulz' else pipeline.CHOLESKY
  kw = dict(inverse_mode=mode, threads_per_env=args.threads_per_env,
            envs_per_cta=args.envs_per_cta)
  rng = np.random.default_rng(1234 + rank)
  q0 = (sys_.init_q + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))).astype(np.float32)
  qd0 = (0.1 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32)
  total = args.warmup + args.steps
  gen = torch.Generator(device=dev)
  gen.manual_seed(77 + rank)
  acts = torch.rand(total, n, sys_.act_size(), device=dev, generator=gen) * 2 - 1
  model = pipeline.model_for(sys_, dev)
  s0 = pipeline.init(sys_, torch.tensor(q0, device=dev), torch.tensor(qd0, device=dev),
                      cache=args.state_cache)
  a_state = s0
  b_state = pipeline._alloc(model, n, False, dev, cache=args.state_cache)
  flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
  stream = torch.cuda.current_stream(dev)

  def one(i, src, dst):
    return pipeline.step(sys_, src, acts[i], n_frames=N_FRAMES, out=dst, **kw)

  for i in range(args.warmup):
    one(i, a_state, b_state)
    a_state, b_state = b_state, a_state
  torch.cuda.synchronize()
  if world > 1:
    dist.barrier()
  torch.cuda.synchronize()
  ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        for _ in range(args.steps)]
  launches = 0
  with ClockSampler(local) as clk:
    for k in range(args.steps):
      flush.zero_()
      ev[k][0].record(stream)
      one(args.warmup + k, a_state, b_state)
      ev[k][1].record(stream)
      launches += _native.lib().braxg_last_launch_count()
      a_state, b_state = b_state, a_state
    torch.cuda.synchronize()
  if world > 1:
    dist.barrier()
  torch.cuda.synchronize()
  times = [a.elapsed_time(b) for a, b in ev]
  t_total = max_over_ranks(sum(times) / 1e3, dev)
  status = a_state.status.cpu().numpy()

  # the same timed loop with the reference's inverse (Newton-Schulz, K = 10)
  other = pipeline.NEWTON_SCHULZ if mode == pipeline.CHOLESKY else pipeline.CHOLESKY
  kw_o = dict(kw, inverse_mode=other)
  c_state = pipeline.init(sys_, torch.tensor(q0, device=dev), torch.tensor(qd0, device=dev),
                      cache=args.state_cache)
  d_state = pipeline._alloc(model, n, False, dev, cache=args.state_cache)
  for i in range(args.warmup):
    pipeline.step(sys_, c_state, acts[i], n_frames=N_FRAMES, out=d_state, **kw_o)
    c_state, d_state = d_state, c_state
  torch.cuda.synchronize()
  t_other = 0.0
  for k in range(args.steps):
    flush.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    pipeline.step(sys_, c_state, acts[args.warmup + k], n_frames=N_FRAMES, out=d_state, **kw_o)
    e1.record(stream)
    c_state, d_state = d_state, c_state
    e1.synchronize()
    t_other += e0.elapsed_time(e1) / 1e3
  t_other = max_over_ranks(t_other, dev)
  other_mode = {'inverse_mode': INVERSE_NAMES['newton_schulz' if other == pipeline.NEWTON_SCHULZ else 'cholesky'],
                'value': round(whole_job_rate(args.steps * n, world, t_other), 1),
                'ms_per_step': round(1e3 * t_other / args.steps, 4)}
  value = whole_job_rate(args.steps * n, world, t_total)
  ms_per_step = 1e3 * t_total / args.steps

  # ---- e2e through the C ABI with host buffers ------------------------------
  # Per step: the actions are copied from pinned host memory, braxg_step runs
  # (called through ctypes with its argument structs built once), and the
  # observation (q, qd) is copied back to pinned host memory and waited for.
  import ctypes
  lib = _native.lib()
  nq_, nv_, nu_ = sys_.q_size(), sys_.qd_size(), sys_.act_size()
  h_act = torch.empty(args.steps, n, nu_, dtype=torch.float32).pin_memory()
  h_act.copy_(acts[args.warmup:].cpu())
  h_q = torch.empty(n, nq_, dtype=torch.float32).pin_memory()
  h_qd = torch.empty(n, nv_, dtype=torch.float32).pin_memory()
  def measure_e2e(mode_, kw_):
    """Env-steps/s of the host-buffer path in one inverse mode."""
    d_act = torch.empty(n, nu_, dtype=torch.float32, device=dev)
    # the same trajectory segment as the device-timed loop: a fresh reset, the
    # same warm-up steps, then the timed steps with the actions read from host
    st = pipeline.init(sys_, torch.tensor(q0, device=dev), torch.tensor(qd0, device=dev),
                        cache=args.state_cache)
    st2 = pipeline._alloc(model, n, False, dev, cache=args.state_cache)
    for k in range(args.warmup):
      pipeline.step(sys_, st, acts[k], n_frames=N_FRAMES, out=st2, **kw_)
      st, st2 = st2, st
    cs = [pipeline._cstate(st), pipeline._cstate(st2)]  # ping-pong: in = cs[k % 2], out = the other
    states = [st, st2]
    c_opt = pipeline._opts(mode_, args.threads_per_env, args.envs_per_cta)
    c_stream = ctypes.c_void_p(stream.cuda_stream)
    torch.cuda.synchronize()
    if world > 1:
      dist.barrier()
    e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(args.steps)]
    api_s = 0.0
    t0 = time.perf_counter()
    for k in range(args.steps):
      e_ev[k][0].record(stream)
      d_act.copy_(h_act[k], non_blocking=True)
      ta = time.perf_counter()
      rc = lib.braxg_step(model.handle, c_stream, n, N_FRAMES, d_act.data_ptr(), ctypes.byref(cs[k % 2]),
                          ctypes.byref(cs[1 - k % 2]), ctypes.byref(c_opt))
      api_s += time.perf_counter() - ta
      if rc != 0:
        _native.check(rc, 'braxg_step')
      out_s = states[1 - k % 2]
      h_q.copy_(out_s.q, non_blocking=True)
      h_qd.copy_(out_s.qd, non_blocking=True)
      e_ev[k][1].record(stream)
      stream.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, dev)
    gpu_e2e = sum(a.elapsed_time(b) for a, b in e_ev) / 1e3
    e2e = {'value': whole_job_rate(args.steps * n, world, t_e2e), 'unit': 'env-steps/s',
           'ms_per_step_wall': round(1e3 * t_e2e / args.steps, 4),
           'ms_per_step_gpu': round(1e3 * gpu_e2e / args.steps, 4),
           'ms_per_step_api_call': round(1e3 * api_s / args.steps, 4),
           'path': 'braxg_step through ctypes; actions H2D from pinned memory, q and qd D2H to pinned memory',
           'h2d_bytes_per_step': n * nu_ * 4,
           'd2h_bytes_per_step': n * (nq_ + nv_) * 4}

    return e2e

  e2e = measure_e2e(mode, kw)
  other_mode['e2e'] = measure_e2e(other, kw_o)

  # ---- roofline -----------------------------------------------------------
  nmv = load_nmv()[WORKLOAD]
  f_step, b_step = algorithmic(sys_, nmv['mean_matvecs_per_step'], args.inverse == 'newton_schulz')
  # the state cache: its position-term spans read at the launch start and
  # written at its end (active constraint rows past the first 32 not counted);
  # overhead traffic of this implementation, not algorithmic bytes
  b_cache = 2 * 4 * model.cache_span[0] if args.state_cache else 0
  b_launch = b_step * n
  launch_s = t_total / args.steps
  flops_launch = f_step * N_FRAMES * n
  achieved = flops_launch / launch_s / 1e12
  props = torch.cuda.get_device_properties(dev)
  peaks = {}
  try:
    with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
      peaks = json.load(f)
  except OSError:
    pass
  sm_max = peaks.get('sm_max_mhz', 2070.0)
  peak_fp32 = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
  hbm_peak = peaks.get('hbm_gbs')
  hbm_src = 'MEASURED_PEAKS.json hbm_gbs (of measured)'
  if hbm_peak is None:
    hbm_peak, hbm_src = 6800.0, 'no MEASURED_PEAKS.json: 6.8 TB/s (of fallback, an earlier GB300 copy measurement)'
  achieved_gbs = b_launch / launch_s / 1e9
  roofline = {
      'bound': 'fp32', 'achieved': round(achieved, 3), 'peak': round(peak_fp32, 1),
      'unit': 'TFLOP/s', 'frac': round(achieved / peak_fp32, 4),
      'traffic': profiled_traffic('step_kernel'),
      'peak_source': (f'nominal FP32 CUDA-core peak ({props.multi_processor_count} SMs x 128 '
                      f'FMA/clk x 2 x {sm_max:.0f} MHz); MEASURED_PEAKS.json has no FP32 figure'),
      'flops_per_launch': flops_launch,
      'hbm': {'achieved_gbs': round(achieved_gbs, 2), 'peak_gbs': hbm_peak,
              'frac': round(achieved_gbs / hbm_peak, 5),
              'algorithmic_bytes_per_launch': b_launch, 'state_bytes_per_env': b_step,
              'overhead': {'cache_bytes_per_env': b_cache, 'cache_bytes_per_launch': b_cache * n,
                           'note': 'position-term cache restore + store: traffic of this design, '
                                   'not algorithmic bytes; included in roofline.traffic'},
              'peak_source': hbm_src},
  }
  clocks = clk.summary()
  adjoint = None if args.no_adjoint else bench_adjoint(torch, pipeline, sys_, dev, rank,
                                                        horizon=args.adjoint_horizon)
  apg_step = None if args.no_adjoint else bench_apg(torch, sys_, dev, rank)
  uneven = None if args.no_uneven else bench_uneven(torch, dev, rank)
  env_step = bench_env(torch, dev, rank)
  humanoid = None if args.no_humanoid else bench_humanoid(torch, pipeline, dev, rank)
  chain3 = bench_chain3(torch, pipeline, dev, rank)
  out = {
      'metric': METRIC, 'value': round(value, 1), 'unit': 'env-steps/s', 'n_gpus': world,
      'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms_per_step, 4),
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
      'data': 'synthetic (seeded resets and U(-1,1) actions)',
      'config': {**workload_config(n, world),
                 'inverse_mode': INVERSE_NAMES[args.inverse],
                 'state_cache': bool(args.state_cache),
                 'l2': 'flushed (256 MB write) before every timed step',
                 'launch_shape': dict(zip(('threads_per_env', 'envs_per_cta', 'smem_bytes'),
                                          model.launch_shape(mode, args.threads_per_env,
                                                             args.envs_per_cta, n_env=n)))},
      'e2e': e2e, 'gpu_launches': launches, 'roofline': roofline, 'clocks': clocks,
      'other_inverse_mode': other_mode,
      'adjoint': adjoint, 'apg_closed_loop': apg_step, 'uneven': uneven, 'env_step': env_step, 'humanoid': humanoid, 'chain3': chain3,
      'env_status_nonzero': int((status != 0).sum()),
      'env_status_bits': status_bits(status),
  }
  if rank == 0 and world == 1 and not args.no_cpu_baseline:
    out['cpu_baseline'] = cpu_baseline(args.cpu_sample_envs)
  if world > 1:
    dist.destroy_process_group()
  if rank == 0:
    print(json.dumps(out))


def bench_adjoint(torch, pipeline, sys_, dev, rank, n=512, horizon=128, ckpt=16, reps=3):
  """Forward rollout vs fused forward + adjoint (the APG workload): quadruped,
  512 envs, 128 env steps of 5 frames, loss -mean(torso x-velocity) +
  1e-3 sum |u|^2, gradients w.r.t. the actions and qd0, checkpoint every 16.
  Timed with every segment's frame snapshots resident (the default when they
  fit: no recompute) and with the smallest workspace (recompute of all but
  the last segment)."""
  rng = np.random.default_rng(55 + rank)
  q0 = torch.tensor((sys_.init_q + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))).astype(np.float32), device=dev)
  qd0 = torch.tensor((0.1 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32), device=dev)
  u = torch.tensor(rng.uniform(-1, 1, (horizon, n, sys_.act_size())).astype(np.float32), device=dev)
  qd_bar = torch.zeros(horizon, n, sys_.qd_size(), device=dev)
  qd_bar[:, :, 0] = -1.0 / horizon
  stream = torch.cuda.current_stream(dev)

  def timed(fn):
    fn()
    torch.cuda.synchronize()
    best = []
    for _ in range(reps):
      e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
      e0.record(stream)
      fn()
      e1.record(stream)
      torch.cuda.synchronize()
      best.append(e0.elapsed_time(e1) / 1e3)
    return statistics.median(best)

  def fwd():
    pipeline.rollout(sys_, pipeline.bare_state(q0, qd0), u, n_frames=N_FRAMES, inverse_mode=pipeline.CHOLESKY,
                     trajectory=True)

  status = [None]

  def fwd_adj(resident=None):
    r = pipeline.rollout_grad(sys_, q0, qd0, u, None, qd_bar, n_frames=N_FRAMES, ckpt_every=ckpt,
                              resident_segments=resident)
    status[0] = r[3]

  def split():  # the custom_vjp shape: forward half, then the reverse half on its residual
    _, tape = pipeline.rollout_vjp_fwd(sys_, q0, qd0, u, n_frames=N_FRAMES, ckpt_every=ckpt)
    pipeline.rollout_vjp_bwd(tape, None, qd_bar)

  def fwd_ns():  # the reference's inverse: the Newton-Schulz rollout from init's exact inverse
    pipeline.rollout(sys_, pipeline.init(sys_, q0, qd0), u, n_frames=N_FRAMES, inverse_mode=pipeline.NEWTON_SCHULZ,
                     trajectory=True)

  def fwd_adj_ns():
    r = pipeline.rollout_grad(sys_, q0, qd0, u, None, qd_bar, n_frames=N_FRAMES, ckpt_every=ckpt,
                              inverse_mode=pipeline.NEWTON_SCHULZ)
    status_ns[0] = r[3]

  status_ns = [None]
  t_f = timed(fwd)
  t_b = timed(fwd_adj)  # every segment's snapshots resident (they fit): no recompute
  t_m = timed(lambda: fwd_adj(1))  # smallest workspace: all but the last segment recomputed
  t_s = timed(split)
  t_fn = timed(fwd_ns)
  t_bn = timed(fwd_adj_ns)
  bad = int((status[0] != 0).sum().item())
  return {'workload': f'quadruped, {n} envs, {horizon} env steps x {N_FRAMES} frames, checkpoint every {ckpt}',
          'fwd_env_steps_per_s': round(n * horizon / t_f, 1),
          'fwd_adj_env_steps_per_s': round(n * horizon / t_b, 1),
          'fwd_ms': round(1e3 * t_f, 3), 'fwd_adj_ms': round(1e3 * t_b, 3),
          'cost_ratio_fwd_adj_over_fwd': round(t_b / t_f, 3),
          'fwd_adj_ms_smallest_workspace': round(1e3 * t_m, 3),
          'cost_ratio_smallest_workspace': round(t_m / t_f, 3),
          'split_fwd_then_bwd_ms': round(1e3 * t_s, 3), 'cost_ratio_split': round(t_s / t_f, 3),
          'newton_schulz': {'fwd_ms': round(1e3 * t_fn, 3), 'fwd_adj_ms': round(1e3 * t_bn, 3),
                            'cost_ratio_fwd_adj_over_fwd': round(t_bn / t_fn, 3),
                            'envs_without_gradient': int((status_ns[0] != 0).sum().item())},
          'envs_without_gradient': bad, 'gpu_launches_fwd_adj': 1}


def bench_apg(torch, sys_, dev, rank, n=512, horizon=32, reps=3):
  """The closed-loop APG training step (brax_gb300/apg.py after
  brax/training/agents/apg/train.py:179-236): an MLP policy acts on each env
  step's observation for `horizon` env steps (5 frames each), one physics
  launch per env step forward and one adjoint launch per env step backward,
  chained by torch.autograd through the policy.  Timed with CUDA events
  around the host loop (the per-step launches and policy calls included):
  the loss alone (no gradient) and the loss plus its backward."""
  from brax_gb300 import apg
  cfg = apg.Config(num_envs=n, horizon=horizon, n_frames=N_FRAMES)
  torch.manual_seed(77 + rank)
  policy = apg.make_policy(sys_.q_size() - 2 + sys_.qd_size(), sys_.act_size(), device=dev)
  rng = np.random.default_rng(78 + rank)
  q0 = torch.tensor((sys_.init_q + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))).astype(np.float32), device=dev)
  qd0 = torch.tensor((0.1 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32), device=dev)
  stream = torch.cuda.current_stream(dev)

  def fwd():
    with torch.no_grad():
      apg.loss(sys_, policy, q0, qd0, cfg)

  def fwd_bwd():
    policy.zero_grad(set_to_none=True)
    apg.loss(sys_, policy, q0, qd0, cfg).backward()

  def timed(fn):
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
      e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
      e0.record(stream)
      fn()
      e1.record(stream)
      torch.cuda.synchronize()
      ts.append(e0.elapsed_time(e1) / 1e3)
    return statistics.median(ts)

  t_f = timed(fwd)
  t_b = timed(fwd_bwd)
  return {'workload': f'closed-loop APG step: quadruped, {n} envs, horizon {horizon} x {N_FRAMES} frames, '
                      f'MLP policy (64, 64), one launch per env step each way',
          'fwd_ms': round(1e3 * t_f, 3), 'fwd_bwd_ms': round(1e3 * t_b, 3),
          'fwd_env_steps_per_s': round(n * horizon / t_f, 1),
          'fwd_bwd_env_steps_per_s': round(n * horizon / t_b, 1),
          'cost_ratio_fwd_bwd_over_fwd': round(t_b / t_f, 3),
          'gpu_launches_fwd_bwd': 2 * horizon}


def bench_env(torch, dev, rank, n=4096, steps=50, warmup=3):
  """The fused env step (locomotion task + EpisodeWrapper + AutoResetWrapper in
  the physics launch) on the headline workload: one launch per env step, L2
  flushed between steps like the pipeline measurement."""
  from brax_gb300 import envs as E
  env = E.Locomotion(WORKLOAD_SYS(), device=dev)
  gen = torch.Generator(device=dev)
  gen.manual_seed(500 + rank)
  st = env.reset(n, generator=gen)
  acts = torch.rand(warmup + steps, n, env.action_size, device=dev, generator=gen) * 2 - 1
  for k in range(warmup):
    st = env.step(st, acts[k])
  flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
  stream = torch.cuda.current_stream(dev)
  torch.cuda.synchronize()
  t = 0.0
  dones = 0.0
  for k in range(steps):
    flush.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    st = env.step(st, acts[warmup + k])
    e1.record(stream)
    e1.synchronize()
    t += e0.elapsed_time(e1) / 1e3
    dones += float(st.done.sum().item())
  bad = int((st.pipeline_state.status != 0).sum().item())
  return {'workload': f'quadruped locomotion task, {n} envs, auto-reset, episode_length 1000, 5 frames',
          'env_steps_per_s': round(steps * n / t, 1), 'ms_per_step': round(1e3 * t / steps, 4),
          'resets_per_env_step': round(dones / steps, 2), 'env_status_nonzero': bad, 'gpu_launches_per_step': 1}


def bench_humanoid(torch, pipeline, dev, rank, n=16384, steps=20, warmup=3):
  """The humanoid-like workload (nv 27, 17 motors, 27 contact slots): 16384
  envs, env step = 5 x 0.003 s, actions N(0, 0.3) clipped to [-1, 1], one
  launch per env step in the bench's default inverse mode, L2 flushed between
  steps."""
  from brax_gb300 import mjcf
  sys_ = mjcf.load_asset('humanoid_like')
  rng = np.random.default_rng(700 + rank)
  q0 = (sys_.init_q + rng.uniform(-0.01, 0.01, (n, sys_.q_size()))).astype(np.float32)
  qa = 3  # the free root's quaternion
  q0[:, qa:qa + 4] /= np.linalg.norm(q0[:, qa:qa + 4], axis=1, keepdims=True)
  qd0 = (0.01 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32)
  gen = torch.Generator(device=dev)
  gen.manual_seed(701 + rank)
  acts = (torch.randn(warmup + steps, n, sys_.act_size(), device=dev, generator=gen) * 0.3).clamp_(-1, 1)
  s = pipeline.init(sys_, torch.tensor(q0, device=dev), torch.tensor(qd0, device=dev))
  model = pipeline.model_for(sys_, dev)
  bufs = [s, pipeline._alloc(model, n, False, dev, cache=True)]
  for k in range(warmup):
    pipeline.step(sys_, bufs[k % 2], acts[k], n_frames=N_FRAMES, inverse_mode=pipeline.CHOLESKY,
                  out=bufs[1 - k % 2])
  flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
  stream = torch.cuda.current_stream(dev)
  torch.cuda.synchronize()
  t = 0.0
  for j in range(steps):
    k = warmup + j
    flush.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    pipeline.step(sys_, bufs[k % 2], acts[k], n_frames=N_FRAMES, inverse_mode=pipeline.CHOLESKY,
                  out=bufs[1 - k % 2])
    e1.record(stream)
    e1.synchronize()
    t += e0.elapsed_time(e1) / 1e3
  last = bufs[(warmup + steps) % 2]
  grad = bench_humanoid_grad(torch, pipeline, sys_, dev, rank)
  return {'workload': f'humanoid-like nq 28 nv 27 nu 17, 27 contact slots, {n} envs, env step = '
                      f'{N_FRAMES} x {sys_.dt} s, actions N(0, 0.3) clipped, Cholesky mode',
          'env_steps_per_s': round(steps * n / t, 1), 'ms_per_step': round(1e3 * t / steps, 4),
          'launch_shape': dict(zip(('threads_per_env', 'envs_per_cta', 'smem_bytes'),
                                   model.launch_shape(pipeline.CHOLESKY, n_env=n))),
          'env_status_nonzero': int((last.status != 0).sum().item()), 'gpu_launches_per_step': 1,
          'gradient': grad}


def bench_humanoid_grad(torch, pipeline, sys_, dev, rank, n=512, horizon=32, ckpt=8, reps=3):
  """APG's gradient on the humanoid-like model (27 dofs, the feet's
  capsule-capsule pair, most solves above 32 rows once it falls): 512 envs,
  32 env steps of 5 frames, loss -mean(torso x-velocity), the fused forward +
  adjoint launch against the plain forward rollout, exact inverse."""
  rng = np.random.default_rng(710 + rank)
  q0 = (sys_.init_q + rng.uniform(-0.01, 0.01, (n, sys_.q_size()))).astype(np.float32)
  q0[:, 3:7] /= np.linalg.norm(q0[:, 3:7], axis=1, keepdims=True)
  q0 = torch.tensor(q0, device=dev)
  qd0 = torch.tensor((0.01 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32), device=dev)
  u = torch.tensor(np.clip(rng.normal(0.0, 0.3, (horizon, n, sys_.act_size())), -1, 1).astype(np.float32),
                   device=dev)
  qd_bar = torch.zeros(horizon, n, sys_.qd_size(), device=dev)
  qd_bar[:, :, 0] = -1.0 / horizon
  stream = torch.cuda.current_stream(dev)
  status = [None]

  def fwd():
    pipeline.rollout(sys_, pipeline.bare_state(q0, qd0), u, n_frames=N_FRAMES, inverse_mode=pipeline.CHOLESKY,
                     trajectory=True)

  def fwd_adj():
    status[0] = pipeline.rollout_grad(sys_, q0, qd0, u, None, qd_bar, n_frames=N_FRAMES, ckpt_every=ckpt)[3]

  def timed(fn):
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
      e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
      e0.record(stream)
      fn()
      e1.record(stream)
      torch.cuda.synchronize()
      ts.append(e0.elapsed_time(e1) / 1e3)
    return statistics.median(ts)

  t_f, t_b = timed(fwd), timed(fwd_adj)
  return {'workload': f'humanoid-like, {n} envs, {horizon} env steps x {N_FRAMES} frames, checkpoint every {ckpt}',
          'fwd_ms': round(1e3 * t_f, 3), 'fwd_adj_ms': round(1e3 * t_b, 3),
          'fwd_adj_env_steps_per_s': round(n * horizon / t_b, 1),
          'cost_ratio_fwd_adj_over_fwd': round(t_b / t_f, 3),
          'envs_without_gradient': int((status[0] != 0).sum().item())}


def bench_chain3(torch, pipeline, dev, rank, n=128, n_steps=1000):
  """The plain 3-link chain workload (nq = nv = 3, no contacts): 128 envs,
  q0 ~ U(-pi/4, pi/4), qd0 ~ N(0, 0.1), zero actions, 1000 pipeline steps of
  0.01 s as one rollout launch (the reference's lax.scan of 1000 steps), in
  both inverse modes.  Its inputs and outputs are a few KB: L2-resident."""
  from brax_gb300 import mjcf
  sys_ = mjcf.load_asset('chain3')
  rng = np.random.default_rng(300 + rank)
  q0 = torch.tensor(rng.uniform(-np.pi / 4, np.pi / 4, (n, 3)).astype(np.float32), device=dev)
  qd0 = torch.tensor(rng.normal(0, 0.1, (n, 3)).astype(np.float32), device=dev)
  acts = torch.zeros(n_steps, n, sys_.act_size(), device=dev)
  stream = torch.cuda.current_stream(dev)
  out = {'workload': f'chain3 (3 hinges, no contact), {n} envs, {n_steps} steps of {sys_.dt} s in one launch'}
  for name, mode in (('exact', pipeline.CHOLESKY), ('newton_schulz', pipeline.NEWTON_SCHULZ)):
    s = pipeline.init(sys_, q0, qd0)
    pipeline.rollout(sys_, s, acts[:10], inverse_mode=mode)  # warm-up
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
      e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
      e0.record(stream)
      last, _ = pipeline.rollout(sys_, s, acts, inverse_mode=mode)
      e1.record(stream)
      torch.cuda.synchronize()
      ts.append(e0.elapsed_time(e1) / 1e3)
    t = statistics.median(ts)
    out[name] = {'env_steps_per_s': round(n * n_steps / t, 1), 'ms_per_rollout': round(1e3 * t, 3),
                 'env_status_nonzero': int((last.status != 0).sum().item())}
  out['gpu_launches_per_rollout'] = 1
  return out


def bench_uneven(torch, dev, rank, total=8192, n_steps=256):
  """The uneven batch: 8192 envs (60 % hinge chains of U{2..32} links with the
  last link against a plane, 25 % quadrupeds, 15 % humanoid-like), 256 env
  steps, shapes from the autotuner; timed as one persistent launch of all 256
  steps and as 256 per-step launches captured in one CUDA graph."""
  from brax_gb300 import autotune, workloads as W
  from brax_gb300.batch import Batch, GraphRollout
  mix = W.uneven_mix(total, seed=rank)
  systems, n_env, n_frames = [m[0] for m in mix], [m[1] for m in mix], [m[2] for m in mix]
  t0 = time.perf_counter()
  shapes = autotune.tune_batch(systems, n_env, n_frames, device=dev)
  tune_s = time.perf_counter() - t0
  tuned = autotune.report(systems, n_env, n_frames, device=dev) or {}
  b = Batch(systems, n_env, n_frames, shapes=shapes, device=dev)
  rng = np.random.default_rng(900 + rank)
  qs, qds, acts = [], [], []
  for s, n, _ in mix:
    q, qd = W.reset(s, n, rng)
    qs.append(q)
    qds.append(qd)
    acts.append(np.stack([W.actions(s, n, rng) for _ in range(n_steps)]).astype(np.float32))
  table = b.concat_steps(acts, 'act')
  s0 = b.init(b.concat(qs, 'q'), b.concat(qds, 'qd'))
  stream = torch.cuda.current_stream(dev)
  out = b.alloc()
  b.rollout(s0, table[:4], out=out)  # warm-up
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  b.rollout(s0, table, out=out)
  e1.record(stream)
  torch.cuda.synchronize()
  t_one = e0.elapsed_time(e1) / 1e3
  bad = int((out.status != 0).sum().item())
  bad_by_family = {}
  for (s, _, _), st in zip(mix, b.split(out.status, 'status')):
    st = st.cpu().numpy()
    k = W.family(s)
    e = bad_by_family.setdefault(k, {'nonfinite': 0, 'not_spd': 0})
    e['nonfinite'] += int(((st & 1) != 0).sum())
    e['not_spd'] += int(((st & 2) != 0).sum())

  def policy(k, state, act):
    act.copy_(table[k])

  g = GraphRollout(b, s0, n_steps, policy)
  for f in ('q', 'qd', 'mass_mx_inv'):
    getattr(g.state, f).copy_(getattr(s0, f))
  torch.cuda.synchronize()
  e0.record(stream)
  g.replay()
  e1.record(stream)
  torch.cuda.synchronize()
  t_graph = e0.elapsed_time(e1) / 1e3
  fam = {}
  for s, n, f in mix:
    k = W.family(s)
    fam[k] = fam.get(k, 0) + n
  return {'workload': f'{total} envs: ' + ', '.join(f'{n} {k}' for k, n in fam.items()) +
                      f' ({len(mix)} models, nv 2-32), {n_steps} env steps (chains 1 frame, others 5)',
          'env_steps_per_s_one_launch': round(total * n_steps / t_one, 1),
          'env_steps_per_s_graph': round(total * n_steps / t_graph, 1),
          'ms_one_launch': round(1e3 * t_one, 3), 'ms_graph': round(1e3 * t_graph, 3),
          'graph_nodes_per_step': 3, 'shapes': shapes, 'launch': b.launch_info(),
          'autotune_s': round(tune_s, 2),
          'autotune': {'candidates_timed': len(tuned.get('timed', {})),
                       'default_ms_16_steps': round(tuned.get('default_ms', float('nan')), 3),
                       'kept_ms_16_steps': round(tuned.get('ms', float('nan')), 3)},
          'env_status_nonzero': bad,
          'env_status_by_family': bad_by_family}


def run_reference(args):
  rank = int(os.environ.get('RANK', '0'))
  world = int(os.environ.get('WORLD_SIZE', '1'))
  if rank != 0:
    return
  ref = CpuReference(args.cpu_sample_envs)
  try:
    value, wall = ref.run(args.steps, args.warmup)
  finally:
    ref.close()
  cb = {'value': value, 'unit': 'env-steps/s', 'cores': ref.cores, 'kind': 'port',
        'sample': ref.describe(args.steps, wall)}
  out = {
      'metric': METRIC, 'value': round(value, 2), 'unit': 'env-steps/s', 'n_gpus': world,
      'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(1e3 * sum(wall) / len(wall), 3),
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
      'impl': 'reference',
      'config': {**workload_config(args.envs, world), 'inverse_mode': 'newton_schulz (the reference algorithm)',
                 'sample': cb['sample']},
      'cpu_baseline': cb,
      'e2e': {'value': round(value, 2), 'unit': 'env-steps/s', 'h2d_bytes_per_step': 0,
              'd2h_bytes_per_step': 0},
      'note': ('the reference is pure Python/JAX and jax/jaxlib/mujoco are not installable here; '
               'this arm times the numpy restatement of the same path (oracle/), kind "port"; '
               'a step is one env step of cores x cpu_sample_envs envs'),
  }
  print(json.dumps(out))


if __name__ == '__main__':
  a = parse()
  if a.impl == 'reference':
    run_reference(a)
  else:
    run_braxg(a)
