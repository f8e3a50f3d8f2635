"""bench.py's multi-GPU mode runs independent replicas (one body per rank, no
collective in the solve): world_size-2 gloo ranks on the CPU check the
rendezvous, the barrier, the max-over-ranks timing and the whole-job value,
and that the reference arm prints only on rank 0."""

import os
import socket
import subprocess
import sys


from conftest import ROOT


def free_port():
  with socket.socket() as s:
    s.bind(('127.0.0.1', 0))
    return s.getsockname()[1]


RANK_SCRIPT = r'''
import os, sys, json
sys.path.insert(0, {root!r})
import bench as B
class A: pass
ws, rank, local = B.dist_init(A())
assert ws == 2 and rank in (0, 1)
B.barrier(ws)
t = 1.0 + rank  # rank 1 is the slow replica
t_max = B.max_over_ranks(ws, t)
print(json.dumps({{'rank': rank, 'max': t_max, 'value': B.replica_value(ws, 10, t_max)}}),
      flush=True)
import torch.distributed as dist
dist.destroy_process_group()
'''


def run_ranks(script, port, extra_env=None):
  procs = []
  for rank in range(2):
    env = dict(os.environ, WORLD_SIZE='2', RANK=str(rank), LOCAL_RANK=str(rank),
               MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES='')
    env.update(extra_env or {})
    procs.append(subprocess.Popen([sys.executable, '-c', script], env=env, stdout=subprocess.PIPE,
                                  stderr=subprocess.PIPE, text=True))
  outs = []
  for p in procs:
    out, err = p.communicate(timeout=240)
    assert p.returncode == 0, err[-2000:]
    outs.append(out)
  return outs


def test_two_replicas_time_by_the_slowest_rank():
  import json
  outs = run_ranks(RANK_SCRIPT.format(root=ROOT), free_port())
  res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
  assert {r['rank'] for r in res} == {0, 1}
  for r in res:
    assert r['max'] == 2.0                      # the slowest replica's time
    assert abs(r['value'] - 2 * 10 / 2.0) < 1e-12  # both ranks' substeps


def test_reference_arm_prints_on_rank_0_only():
  """`bench.py --impl reference` under two ranks: rank 1 exits at once
  without output; rank 0's CPU sample is skipped here by running rank 1
  alone (the sample itself is covered by the CPU port tests)."""
  env = dict(os.environ, WORLD_SIZE='2', RANK='1', LOCAL_RANK='1', MASTER_ADDR='127.0.0.1',
             MASTER_PORT=str(free_port()), CUDA_VISIBLE_DEVICES='')
  r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference',
                      '--gpus', '2', '--steps', '1', '--warmup', '0'], env=env,
                     capture_output=True, text=True, timeout=240)
  assert r.returncode == 0, r.stderr[-2000:]
  assert r.stdout.strip() == ''
