"""Shared helpers for the GPU parity tests (kernel vs oracle).

oracle_check is the parity bar of tests/test_gpu_bench_parity.py (its
module docstring states it), shared with the other tests that compare one or
a few pipeline steps against the oracle."""

import numpy as np

from brax_gb300 import mjcf

WORKLOADS = ('chain3', 'quadruped', 'humanoid_like')


def seeded_inputs(sys, n, seed=0):
  """Reset distribution of the workloads: q jitter U(-0.1, 0.1) on init_q
  (brax/envs/ant.py:209-213), qd ~ 0.1 N(0, 1); the chain uses
  q0 ~ U(-pi/4, pi/4), qd0 ~ N(0, 0.1)."""
  rng = np.random.default_rng(seed)
  if sys.name == 'chain3' or sys.name.startswith('chain'):
    q = rng.uniform(-np.pi / 4, np.pi / 4, (n, sys.q_size()))
    qd = rng.normal(0, 0.1, (n, sys.qd_size()))
  else:
    q = sys.init_q + rng.uniform(-0.1, 0.1, (n, sys.q_size()))
    qd = 0.1 * rng.normal(size=(n, sys.qd_size()))
  return q, qd


def actions(sys, n, rng):
  if sys.name == 'humanoid_like':
    return np.clip(rng.normal(0, 0.3, (n, sys.act_size())), -1, 1)
  if sys.name == 'chain3':
    return np.zeros((n, sys.act_size()))
  return rng.uniform(-1, 1, (n, sys.act_size()))


def rel_err(a, b):
  """Per-env relative error: max |a - b| / max(max |b|, 1) over the trailing axes."""
  a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
  b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
  return np.abs(a - b).max(-1) / np.maximum(np.abs(b).max(-1), 1.0)


def load(name):
  return mjcf.load_asset(name)


# draws of the FP32 rounding envelope: (seed, bias, order) of
# oracle.pipeline.Oracle's perturbation; the two biased draws take every
# near-tie decision one way and the other, three more at random, and three
# evaluate the dense products whose terms cancel (J Minv J^T, J Minv
# qf_smooth, Minv qf, the inverse) in another exact FP32 order without other
# perturbation
ENVELOPE_DRAWS = ((1000, -1, 'reference'), (1001, 1, 'reference'), (1002, 0, 'reference'),
                  (1003, 0, 'reference'), (1004, 0, 'reference'), (None, 0, 'right'), (None, 0, 'rounded'),
                  (None, 0, 'fma'))


def oracle_check(sys, q, qd, minv, act, n_frames, exact, got_q, got_qd, label, strict=False):
  """n_frames pipeline steps of the FP32 and FP64 oracles from the GPU's FP32
  inputs; asserts the bar of this module on the GPU's q / qd (strict: a
  single pipeline step, the 1e-5 p99 bar and the per-env bound; else the
  whole env step's p99 bars) and returns the stats."""
  from oracle.pipeline import Oracle
  mi = None if exact else minv
  act32 = act.astype(np.float32)
  o32 = Oracle(sys, np.float32, exact_inverse=exact)
  o64 = Oracle(sys, np.float64, exact_inverse=exact)
  r32 = o32.env_step(o32.restore(q, qd, mi), act32, n_frames)
  r64 = o64.env_step(o64.restore(q.astype(np.float64), qd.astype(np.float64),
                                 None if exact else minv.astype(np.float64)),
                     act.astype(np.float64), n_frames)
  spread = {'q': np.zeros(q.shape[0]), 'qd': np.zeros(q.shape[0])}
  for seed, bias, order in ENVELOPE_DRAWS:
    op = Oracle(sys, np.float32, exact_inverse=exact, perturb_seed=seed, perturb_bias=bias, order=order)
    rp = op.env_step(op.restore(q, qd, mi), act32, n_frames)
    for f in spread:
      spread[f] = np.maximum(spread[f], rel_err(getattr(rp, f), getattr(r32, f)))
  stats = {}
  for f, g in (('q', got_q), ('qd', got_qd)):
    e32 = rel_err(g, getattr(r32, f))
    e64 = rel_err(g, getattr(r64, f))
    eo = rel_err(getattr(r32, f), getattr(r64, f))
    env = np.maximum(spread[f], eo)
    p99 = lambda x: float(np.quantile(x, 0.99))
    st = {'gpu_vs_fp32_p50': float(np.median(e32)), 'gpu_vs_fp32_p99': p99(e32), 'gpu_vs_fp32_max': float(e32.max()),
          'gpu_vs_fp64_p99': p99(e64), 'fp32_oracle_vs_fp64_p99': p99(eo), 'envelope_p99': p99(env),
          'within_1e-5': float((e32 <= 1e-5).mean())}
    stats[f] = st
    print(f'{label} {f}: vs fp32 p50 {st["gpu_vs_fp32_p50"]:.2e} p99 {st["gpu_vs_fp32_p99"]:.2e} '
          f'max {st["gpu_vs_fp32_max"]:.2e} ({100 * st["within_1e-5"]:.2f}% <= 1e-5) | vs fp64 p99 '
          f'{st["gpu_vs_fp64_p99"]:.2e} (fp32 oracle {st["fp32_oracle_vs_fp64_p99"]:.2e}) | fp32 envelope p99 '
          f'{st["envelope_p99"]:.2e}')
    out = np.nonzero(e32 > 1e-5)[0]
    for i in out[np.argsort(-e32[out])][:12]:
      print(f'  env {i}: vs fp32 {e32[i]:.2e}, fp32 envelope {env[i]:.2e} (perturbed {spread[f][i]:.2e}, '
            f'fp32 oracle vs fp64 {eo[i]:.2e}), vs fp64 {e64[i]:.2e}')
    if strict:
      # per env: within its own envelope, or within the model's FP32 accuracy
      bad = e32 > np.maximum(max(1e-5, 3 * st['fp32_oracle_vs_fp64_p99']), 10 * env)
      assert not bad.any(), (label, f, np.nonzero(bad)[0][:10], e32[bad][:10], env[bad][:10])
      # envs whose FP32 result is determined to 1e-5 (envelope <= 1e-5)
      det = env <= 1e-5
      st['determined'] = float(det.mean())
      st['gpu_vs_fp32_p99_determined'] = p99(e32[det]) if det.any() else 0.0
      print(f'  {100 * st["determined"]:.2f}% of envs determined to 1e-5 in FP32: vs fp32 p99 '
            f'{st["gpu_vs_fp32_p99_determined"]:.2e}')
      # 1e-5, or the FP32 reference path's own accuracy on an ill-conditioned model
      assert st['gpu_vs_fp32_p99_determined'] <= max(1e-5, 1.5 * st['fp32_oracle_vs_fp64_p99']), (label, f, st)
    else:
      bar = max(1e-5, 2 * st['envelope_p99'])
      assert st['gpu_vs_fp32_p99'] <= bar, (label, f, st)
      assert st['gpu_vs_fp64_p99'] <= bar, (label, f, st)
  return stats
