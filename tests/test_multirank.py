"""The N > 1 host path of bench.py on CPU: two gloo ranks (127.0.0.1), each a
replica with its own seeds, reduce their timings with one all-reduce MAX and
report whole-job throughput over the slowest rank."""

import os
import socket

import pytest

torch = pytest.importorskip('torch')


def _free_port():
  with socket.socket() as s:
    s.bind(('127.0.0.1', 0))
    return s.getsockname()[1]


def _rank(rank, world, port, out):
  import torch.distributed as dist
  os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                    WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
  dist.init_process_group('gloo', rank=rank, world_size=world)
  import bench
  t = bench.max_over_ranks(1.0 + rank, 'cpu')       # rank r "took" 1 + r seconds
  rate = bench.whole_job_rate(4096 * 10, world, t)   # 10 steps of 4096 envs per replica
  cfg = bench.workload_config(4096, world)
  out.put((rank, t, rate, cfg['parallelism']))
  dist.barrier()
  dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
  ctx = torch.multiprocessing.get_context('spawn')
  q = ctx.Queue()
  port = _free_port()
  procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
  for p in procs:
    p.start()
  res = sorted(q.get(timeout=120) for _ in procs)
  for p in procs:
    p.join(timeout=60)
    assert p.exitcode == 0
  for rank, t, rate, par in res:
    assert t == 2.0                      # both ranks see the slowest rank's time
    assert rate == 4096 * 10 * 2 / 2.0   # whole-job units over that time
    assert par == 'replicas x2'


def test_single_rank_needs_no_process_group():
  import bench
  assert bench.max_over_ranks(3.5, 'cpu') == 3.5


def test_reference_arm_runs_on_rank_0_only(monkeypatch, capsys):
  """Under torchrun the reference arm's other ranks exit without work: no
  worker pool, no output line."""
  import bench
  monkeypatch.setenv('RANK', '1')
  monkeypatch.setenv('WORLD_SIZE', '2')
  monkeypatch.setattr(bench, 'CpuReference', lambda *a, **k: pytest.fail('rank 1 started the CPU pool'))
  bench.run_reference(bench.parse(['--impl', 'reference', '--steps', '1', '--warmup', '0']))
  assert capsys.readouterr().out == ''


def test_reference_arm_line(monkeypatch, capsys):
  """Rank 0's reference line: the contract's keys, e2e with no host-device
  bytes, and a cpu_baseline describing this run (a stub pool)."""
  import json
  import bench

  class Stub:
    cores = 4

    def __init__(self, n):
      self.sample_envs = n

    def run(self, steps, warmup):
      return 1234.5, [0.1] * steps

    def describe(self, steps, wall):
      return f'stub {steps}'

    def close(self):
      pass

  monkeypatch.setenv('RANK', '0')
  monkeypatch.setenv('WORLD_SIZE', '1')
  monkeypatch.setattr(bench, 'CpuReference', Stub)
  bench.run_reference(bench.parse(['--impl', 'reference', '--steps', '3', '--warmup', '1']))
  d = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
  assert d['impl'] == 'reference' and d['value'] == 1234.5 and d['steps'] == 3 and d['warmup'] == 1
  assert d['e2e'] == {'value': 1234.5, 'unit': 'env-steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
  assert d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['cores'] == 4
  assert d['higher_is_better'] is True and d['unit'] == 'env-steps/s'
