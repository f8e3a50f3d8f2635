#!/usr/bin/env python3
"""MGPBD substeps/sec on GB300 (one JSON line on stdout).

Workload (one "step" = one MGPBD substep = prediction + Newton/PCG solve +
velocity update): a 40x40x40 hex cube, 5 tets per hex (68,921 vertices,
320,000 tets), rest shape the regular grid, start positions jittered
U(+-0.01 h) from seed 0, unit vertex mass, top face pinned (kinematic),
gravity -9.8, dt = 1/60 / 5 substeps, compliance drawn log-uniform in
[1e-9, 1e-4] from the seed (alpha~ = compliance / dt^2), PCG to relative
residual 1e-6.  Constraints (--constraints): by default one length
constraint per unique tet edge plus one volume constraint (det F - 1) per
tet, the construction the benchmark configuration names (718,520
constraints, 72.4M level-0 nonzeros); 'arap' is the reference step's one
ARAP constraint per tet (25.9M nonzeros), also reported as a secondary leg.
Synthetic data: the reference's experiment meshes are not available.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--constraints edge_volume|arap] [--workload cube|slab]

`--workload slab` prints the stiff-drag slab's line instead: 100x100x25
hexes (1.25 M tets), compliance 1e-10, one long edge pinned, the opposite
corner dragged 0.5 along +z over 60 frames; fast step only.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = 'MGPBD substeps/sec @ rel-res 1e-6: learned+mixed+batched vs plain FP32 AMG-PCG'
UNIT = 'substeps/s'


def peaks():
  p = os.path.join(HERE, 'MEASURED_PEAKS.json')
  if os.path.exists(p):
    d = json.load(open(p))
    return float(d['hbm_gbs']), 'measured'
  return 6800.0, 'fallback'


def workload(n, seed=0):
  from controllable_pbd_3d_gb300.scenarios import cube_body
  return cube_body(n, seed)


# CG runs to relative residual 1e-6 (the cap is never reached on this
# workload: ~2,500 iterations per solve for the plain AMG-PCG, ~760 per
# substep for the fast step)
SOLVER_KW = dict(damp=1.0, maxiter=20, atol=1e-4, rtol=1e-2, maxiter_cg=6000, tol_cg=1e-12,
                 rel_tol_cg=1e-6, n_smooth=2, kinematic_pins=True)
# the optimised step: each CG solve is one cooperative persistent kernel on
# the dual system, preconditioned by a degree-8 Chebyshev polynomial in A
# itself (matrix-free operator; no Jacobi scaling, which would spread the
# single alpha~ eigenvalue of the null space of J^T); the operator data is
# staged in shared memory where a block's share fits, as for the ARAP body,
# and read through L2 otherwise, as for the length + volume body; the first
# solve of each substep starts from the previous substep's solution (the
# reference starts every solve from 0)
FAST_KW = dict(mode='fast', precond='cheb', cheb_degree=8, cheb_lo=1e-3, cheb_scale='none',
               primal=False, warm_substep=True)
# the plain float32 AMG-PCG: the reference's two-level tet-aggregation V-cycle
# PCG on CSR matrices (smoother weight capped at 4/(3 lambda_max) because
# omega = 2/3 diverges at this stiffness), each CG solve one CUDA graph with
# a device-side WHILE loop (no host round trip per CG iteration)
PLAIN_KW = dict(mode='fast', smoother='safe', precond='vcycle')
DT = 1.0 / 60.0 / 5.0


class ClockSampler:
  """nvidia-smi clocks/throttle reasons sampled during the timed region."""

  def __init__(self, index=0):
    self.index = index
    self.proc = None
    self.lines = []

  def __enter__(self):
    try:
      self.proc = subprocess.Popen(
          ['nvidia-smi', f'--id={self.index}',
           '--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,'
           'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
           'clocks_event_reasons.sw_power_cap', '--format=csv,noheader,nounits', '-lms', '100'],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
      self.t = threading.Thread(target=self._read, daemon=True)
      self.t.start()
    except (OSError, FileNotFoundError):
      self.proc = None
    return self

  def _read(self):
    for ln in self.proc.stdout:
      self.lines.append(ln.strip())

  def __exit__(self, *a):
    if self.proc is not None:
      self.proc.terminate()
      try:
        self.proc.wait(timeout=5)
      except subprocess.TimeoutExpired:
        self.proc.kill()

  def summary(self):
    sm, mx, reasons = [], [], set()
    names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
    for ln in self.lines:
      f = [x.strip() for x in ln.split(',')]
      if len(f) < 6:
        continue
      try:
        sm.append(float(f[0]))
        mx.append(float(f[1]))
      except ValueError:
        continue
      for name, v in zip(names, f[2:6]):
        if v.lower().startswith('active'):
          reasons.add(name)
    if not sm:
      return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
    return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(mx), 'reasons': sorted(reasons),
            'samples': len(sm)}


def dist_init(args):
  ws = int(os.environ.get('WORLD_SIZE', '1'))
  rank = int(os.environ.get('RANK', '0'))
  local = int(os.environ.get('LOCAL_RANK', '0'))
  import torch
  if ws > 1:
    import torch.distributed as dist
    dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
  return ws, rank, local


def barrier(ws):
  if ws > 1:
    import torch.distributed as dist
    dist.barrier()


def max_over_ranks(ws, v):
  if ws == 1:
    return v
  import torch
  import torch.distributed as dist
  dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
  t = torch.tensor([v], dtype=torch.float64, device=dev)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def replica_value(ws, steps, t_max):
  """Whole-job substeps/s of ws independent replicas that each ran
  `steps` substeps: all replicas' substeps over the slowest replica's time
  t_max (weak scaling)."""
  return ws * steps / t_max


CONSTRAINT_NAMES = {'edge_volume': 'one length constraint per tet edge + one volume '
                                   'constraint (det F - 1) per tet',
                    'arap': 'one ARAP constraint per tet (the reference step)'}


def bench_config(args, ws, n_verts, n_tets, n_cons, nnz0, compliance):
  """The workload's description, the same dict in both arms."""
  return {'workload': f'{args.size}^3 hex cube, 5 tets/hex', 'n_verts': int(n_verts),
          'n_tets': int(n_tets), 'constraints': CONSTRAINT_NAMES[args.constraints],
          'n_constraints': int(n_cons), 'nnz_level0': int(nnz0), 'compliance': compliance,
          'dt': DT, 'rel_res_cg': 1e-6,
          'l2': 'GPU arm: flushed between timed substeps (256 MB write, inside the timed region)',
          'parallelism': f'replicas{ws}'}


def make_solver(torch, n, kw, constraints='edge_volume'):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xr, x0, t, invm, compliance = workload(n)
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], DT,
                     compliance=compliance, constraints=constraints, **kw)
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  s.init()
  torch.cuda.synchronize()
  s.init_s = time.perf_counter() - t0
  return s, x, compliance


L2_FLUSH_BYTES = 256 << 20  # > the 129 MB L2


def time_steps(torch, s, k, first, flush=None):
  """k substeps between CUDA events; with `flush` (a device buffer larger
  than L2) the buffer is overwritten after every substep, inside the timed
  region, so no substep starts with the previous one's data in L2."""
  stream = torch.cuda.current_stream()
  st = []
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  torch.cuda.synchronize()
  e0.record(stream)
  for i in range(k):
    s.step(first + i)
    st.append(s.stats())
    if flush is not None:
      flush.fill_(i)
  e1.record(stream)
  torch.cuda.synchronize()
  return e0.elapsed_time(e1) / 1e3, st


def _event_time(torch, fn, reps):
  """Average device time of fn's launches: `reps` calls captured into one
  CUDA graph (so host launch overhead does not leave gaps), replayed once
  between CUDA events on the stream the kernels run on."""
  for _ in range(3):
    fn()
  torch.cuda.synchronize()
  g = torch.cuda.CUDAGraph()
  side = torch.cuda.Stream()
  with torch.cuda.stream(side):
    with torch.cuda.graph(g, stream=side):
      for _ in range(reps):
        fn()
  torch.cuda.synchronize()
  stream = torch.cuda.current_stream()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  g.replay()
  torch.cuda.synchronize()
  e0.record(stream)
  g.replay()
  e1.record(stream)
  torch.cuda.synchronize()
  return e0.elapsed_time(e1) / 1e3 / reps


def roofline_matrix_free(torch, s, hbm_peak, peak_kind, reps=50):
  """Matrix-free A x as two stand-alone launches (vertex phase + tet
  phase), timed with CUDA events on the current stream; bytes from
  apply_bytes."""
  nt, nv = s.n_tets, s.n_verts
  x = torch.randn(nt, device='cuda')
  s.apply_A(x, matrix_free=1)
  dt = _event_time(torch, lambda: s.apply_A(x, matrix_free=2), reps)
  ne, _ = operator_shape(s)
  bytes_ = apply_bytes(nt, nv, ne, 0)  # the per-phase tet kernel reads all four slots
  achieved = bytes_ / dt / 1e9
  return {'kernel': 'k_jv<kSrcX> + k_jt_plain (matrix-free A x, 2 launches)', 'bound': 'hbm',
          'achieved': round(achieved, 1), 'peak': hbm_peak, 'unit': 'GB/s',
          'frac': round(achieved / hbm_peak, 4), 'peak_kind': peak_kind,
          'algorithmic_bytes_per_launch': bytes_, 'launch_us': round(dt * 1e6, 2),
          'working_set_note': 'operator data of repeated applications stays partly in the '
                              '129 MB L2, so the rate can exceed the HBM roofline',
          'traffic': None}


def apply_bytes(nt, nv, ne=None, n2=0):
  """Algorithmic bytes of one matrix-free A x over nt constraints, ne
  vertex-incidence entries (4 per constraint, 2 per length constraint) and
  n2 length constraints read in compact form: the vertex phase reads the
  vertex-major gradients (16 B per entry), row offsets and inverse masses,
  gathers x once per constraint and writes u (16 B per vertex); the tet
  phase reads constraint indices and gradients (16 + 48 B, compact length
  constraints 8 + 16 B), alpha, x, gathers u once per vertex and writes y."""
  ne = 4 * nt if ne is None else ne
  return (16 * ne + 4 * (nv + 1) + 4 * nv + 4 * nt + 16 * nv) + \
         (64 * (nt - n2) + 24 * n2 + 16 * nv + 4 * nt + 4 * nt + 4 * nt)


def cg_iteration_bytes(nt, nv, degree, ne=None, n2=0):
  """Algorithmic bytes of one Chebyshev-preconditioned CG iteration of the
  persistent kernel: `degree` operator applications, plus per constraint
  the Chebyshev-step vectors (r, d, 1/diag read, d, z written: 20 B per step
  after the first), the p / Ap phase (z, p read, p, Ap written: 16 B) and the
  x / r update (p, Ap, x, x-compensation, r, 1/diag read; x,
  x-compensation, r, z, d written: 44 B)."""
  return degree * apply_bytes(nt, nv, ne, n2) + (degree - 1) * 20 * nt + 16 * nt + 44 * nt


def primal_iteration_bytes(nt, nv, degree, ne=None, n2=0):
  """Algorithmic bytes of one primal (vertex-space) CG iteration: `degree`
  applications of K, each a tet phase (constraint indices 16 B and
  gradients 48 B, compact length constraints 8 + 16 B; alpha 4 B, s written
  4 B, the vertex vector gathered once per vertex 16 B) and a vertex phase
  (vertex-major gradients 16 B per incidence entry, offsets and weights 8 B
  per vertex, s gathered once per constraint); per vertex the Chebyshev
  epilogue (z, r, d, 3x3 inverse read, d, z written: 112 B) in every step
  after the first, the first tet phase's extra p and r gathers (32 B), the
  p / Kp epilogue (64 B) and the y / r update (192 B)."""
  ne = 4 * nt if ne is None else ne
  per_apply = 72 * (nt - n2) + 32 * n2 + 16 * ne + 4 * nt + 24 * nv
  return degree * per_apply + (degree - 1) * 112 * nv + (32 + 64 + 192) * nv


def operator_shape(s):
  """(incidence entries, length constraints) of a solver's operator: a
  length constraint contributes 2 incidence entries instead of 4."""
  n2 = 0 if s.constraint_types is None else int((s.constraint_types == 1).sum())
  return 4 * (s.n_tets - n2) + 2 * n2, n2


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per CG iteration
# of the dual persistent kernel on the 40^3 length + volume workload, from one
# ncu capture of one launch of `bench.py --profile-solve --size 40` (461 CG
# iterations, 56.87 GB; the unscaled Chebyshev-8 polynomial of the headline).
# A launch's traffic is this times its iterations.
TRAFFIC_PER_IT_40 = {'edge_volume': {'k_jcg': 56.87e9 / 461}}
TRAFFIC_SOURCE = {
    'edge_volume': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of bench.py '
                   '--profile-solve --size 40 (461 CG iterations, 56.87 GB), per iteration x '
                   'this launch\'s iterations'}


def roofline_from_steps(st, nt, nv, degree, hbm_peak, peak_kind, size=40, constraints='arap',
                        shape=(None, 0)):
  """Roofline of the two persistent kernels over the timed steps, from the
  CUDA events the library records around each launch on its stream (stats
  ms_warm / ms_dual) and the iterations each ran.  The one with more GPU
  time is returned, the other under 'other'.  Both keep the operator on
  chip (shared memory / L2), so achieved is an on-chip rate."""
  ms_w = sum(x['ms_warm'] for x in st)
  ms_d = sum(x['ms_dual'] for x in st)
  it_w = sum(x['cg_iters_warm'] for x in st)
  it_d = sum(x['cg_iters_total'] for x in st) - it_w
  launches = sum(x['cg_launches'] for x in st)
  n_w = sum(x['newton_iters'] for x in st) if it_w else 0
  n_d = launches - n_w
  path = st[-1]['cg_path']
  ne, n2 = shape
  # staged kernels read every constraint's four slots in the tet phase; the
  # unstaged ones take the length constraints in compact form
  n2 = 0 if path.endswith('staged') else n2
  out = []
  for name, ms, its, n, per_it in (
      (f'k_pcg<{int(path.endswith("staged"))}> (primal warm start, persistent Chebyshev-{degree} '
       'CG on K)', ms_w, it_w, n_w, primal_iteration_bytes(nt, nv, degree, ne, n2)),
      (f'k_jcg<{int(path.endswith("staged"))}> (dual persistent Chebyshev-{degree} CG on A)',
       ms_d, it_d, n_d, cg_iteration_bytes(nt, nv, degree, ne, n2))):
    if n <= 0 or ms <= 0:
      continue
    dt = ms / 1e3 / n
    bytes_ = per_it * its / n
    achieved = bytes_ / dt / 1e9
    out.append({'kernel': name, 'bound': 'hbm', 'achieved': round(achieved, 1),
                'peak': hbm_peak, 'unit': 'GB/s', 'frac': round(achieved / hbm_peak, 4),
                'peak_kind': peak_kind, 'algorithmic_bytes_per_launch': int(bytes_),
                'bytes_per_cg_iteration': per_it, 'launches': n,
                'cg_iterations_per_launch': round(its / n, 1), 'launch_us': round(dt * 1e6, 1),
                'us_per_cg_iteration': round(ms * 1e3 / max(its, 1), 2),
                'share_of_step_gpu_time': None,
                'traffic': (int(TRAFFIC_PER_IT_40[constraints][name[:5]] * its / n)
                            if size == 40 and name[:5] in TRAFFIC_PER_IT_40.get(constraints, {})
                            else None)})
  out.sort(key=lambda r: -r['launch_us'] * r['launches'])
  total = sum(r['launch_us'] * r['launches'] for r in out)
  for r in out:
    r['share_of_cg_gpu_time'] = round(r['launch_us'] * r['launches'] / total, 3)
    del r['share_of_step_gpu_time']
  roof = dict(out[0])
  roof['cg_path'] = path
  if roof['traffic'] is not None:
    roof['traffic_source'] = TRAFFIC_SOURCE[constraints]
  if path.endswith('staged'):
    roof['working_set_note'] = ('operator data staged in shared memory / resident in L2 across '
                                'each solve: the rate is on-chip, not HBM')
  else:
    roof['working_set_note'] = ('operator read from L2 / HBM each application (too large to '
                                'stage in shared memory); part of it stays in the 129 MB L2')
  if roof['traffic'] is not None:
    roof['traffic_over_algorithmic'] = round(roof['traffic'] /
                                             max(roof['algorithmic_bytes_per_launch'], 1), 4)
    # the DRAM rate itself (ncu bytes over the same launch time): most of the
    # algorithmic bytes are served by L2, so this is far below `frac`
    dram_gbs = roof['traffic'] / (roof['launch_us'] * 1e-6) / 1e9
    roof['dram_gbs'] = round(dram_gbs, 1)
    roof['dram_frac'] = round(dram_gbs / hbm_peak, 4)
  if len(out) > 1:
    roof['other'] = out[1]
  return roof


def roofline_csr(torch, s, hbm_peak, peak_kind, reps=40):
  """Level-0 weighted Jacobi sweep of the CSR V-cycle (the dominant launch
  of the plain AMG-PCG: 4 per CG iteration) and the level-0 SpMV, both the
  vectorised row kernel, timed with CUDA events (launches captured into a
  CUDA graph; the 207 MB matrix does not fit in L2)."""
  A = s._gpu_solver._gpu_As[0]
  n, nnz = A.n_rows, A.nnz
  b = torch.randn(n, device='cuda')
  x = torch.randn(n, device='cuda')
  y = torch.empty_like(x)
  out = {}
  for name, f, extra in (
      ('jacobi', lambda: s.level_sweep(0, 1, x, b, y, 0.5), 4 * n * 4),
      ('spmv', lambda: s.level_sweep(0, 0, x, None, y), 4 * n * 2)):
    dt = _event_time(torch, f, reps)
    # algorithmic bytes: values + column ids + row pointers, plus x gathered
    # once, y written (and b, 1/diag read for the sweep)
    bytes_ = 8 * nnz + 4 * (n + 1) + extra
    achieved = bytes_ / dt / 1e9
    out[name] = {'bound': 'hbm', 'achieved': round(achieved, 1), 'peak': hbm_peak, 'unit': 'GB/s',
                 'frac': round(achieved / hbm_peak, 4), 'peak_kind': peak_kind,
                 'algorithmic_bytes_per_launch': bytes_, 'launch_us': round(dt * 1e6, 2),
                 'traffic': None}
  code = s.row_shape(0) or 406
  g, u = divmod(code, 100)
  roof = dict(out['jacobi'])
  roof['kernel'] = f'k_csr_rows_vec<{g},{u},kJacobi> (level-0 weighted Jacobi sweep, CSR)'
  roof['spmv'] = dict(out['spmv'], kernel=f'k_csr_rows_vec<{g},{u},kSpmv> (level-0 SpMV, CSR)')
  return roof


def cpu_model():
  """The host CPU's model name (lscpu, else /proc/cpuinfo), for the record."""
  try:
    out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
    for ln in out.splitlines():
      if ln.lower().startswith('model name'):
        return ln.split(':', 1)[1].strip()
  except (OSError, subprocess.SubprocessError):
    pass
  try:
    for ln in open('/proc/cpuinfo'):
      if ln.lower().startswith(('model name', 'cpu part')):
        return ln.split(':', 1)[1].strip()
  except OSError:
    pass
  return 'unknown'


# CG iteration cap of the CPU substeps: far above what a solve to 1e-6 takes
# on this workload (~2,500-3,000), so it never decides a timing
CPU_MAXITER_CG = 100000
# seconds of whole CPU substeps the CPU legs time (at least one substep)
CPU_BUDGET_S = 120.0


class CpuSubsteps:
  """Whole substeps of the plain MGPBD step on the host cores: the OpenMP
  CPU port of the reference algorithm (oracle/cpu_step.cpp, all host
  threads) on the same workload.  A substep is the prediction, every Newton
  iteration (constraints, residual, matrix fill, Galerkin refill, smoother
  weights, V-cycle PCG to relative residual 1e-6, scatter, line search,
  apply) until the Newton test holds, and the velocity update.  The
  constraint set, its CSR pattern, the tet aggregation and the Galerkin
  structure come from the oracle's restatement (oracle/mgpbd_oracle.py);
  no library of the product is loaded."""

  def __init__(self, n, constraints='edge_volume'):
    from oracle import mgpbd_oracle as MO
    from oracle.cpu_port import CpuPort, threads
    xr, x0, t, invm, compliance = workload(n)
    ctype = agg = None
    t0 = time.perf_counter()
    if constraints == 'edge_volume':
      c, ctype, _, _ = MO.edge_volume_system(t)
      aggs, _ = MO.edge_volume_hierarchy(t)
      agg = aggs[0] if aggs else None
      t = c
    self.port = CpuPort(x0, xr, invm, t, [0.0, -9.8, 0.0], DT, compliance=compliance,
                        maxiter=SOLVER_KW['maxiter'], atol=SOLVER_KW['atol'],
                        rtol=SOLVER_KW['rtol'], maxiter_cg=CPU_MAXITER_CG,
                        tol_cg=SOLVER_KW['tol_cg'], rel_tol_cg=SOLVER_KW['rel_tol_cg'],
                        n_smooth=SOLVER_KW['n_smooth'], kinematic_pins=True, ctype=ctype,
                        hierarchy=agg)
    self.setup_s = time.perf_counter() - t0
    self.threads = threads()

  def run(self, max_steps, budget_s):
    """Time whole substeps, one after another from substep 0, until
    max_steps are done or the time spent reaches budget_s (at least one).
    Returns (seconds per substep, substeps timed, Newton iterations and CG
    iterations per substep)."""
    times, newton, cg = [], [], []
    while len(times) < max(1, max_steps):
      t0 = time.perf_counter()
      self.port.step()
      times.append(time.perf_counter() - t0)
      log = self.port.log  # one row per residual check; solves have PCG time
      newton.append(sum(1 for r in log if r[5] > 0))
      cg.append(sum(r[1] for r in log))
      if sum(times) >= budget_s:
        break
    k = len(times)
    return sum(times) / k, k, sum(newton) / k, sum(cg) / k


def cpu_line(sub, per_step, k, newton, cg):
  return {'value': round(1.0 / per_step, 6), 'unit': UNIT, 'cores': sub.threads, 'kind': 'port',
          'cpu_model': cpu_model(),
          'sample': f'{k} whole substep(s) from substep 0, timed one by one: {newton:g} Newton '
                    f'iterations and {cg:.0f} CG iterations (V-cycle PCG to relative residual '
                    f'1e-6) per substep, {per_step:.1f} s each; OpenMP CPU port of the plain '
                    f'step (oracle/cpu_step.cpp), {sub.threads} host threads; structure built by '
                    f'the oracle in {sub.setup_s:.1f} s (not timed)'}


def net_forward_bytes(n, nnz):
  """Algorithmic bytes of one weights pass of the coarse network: layer 1
  (CSR row: indptr, column, value; 1/diag and field of each neighbour; the
  scaled value written; 64 bf16 features written) and two fused layers
  (column + scaled value per nonzero, the neighbour's 64 bf16 features per
  nonzero, own features read and written), plus the field and norm passes."""
  l1 = 4 * (n + 1) + nnz * (4 + 4 + 4 + 4 + 4) + n * (4 + 128)
  layer = nnz * (4 + 4 + 128) + n * (128 + 128)
  return l1 + 2 * layer + n * 16


LEARNED_TRAIN_BODIES = 12


def learned_leg(torch, args, hbm, kind, plain=None):
  """The learned coarse correction, trained off-body: pairs recorded by
  the plain solver on LEARNED_TRAIN_BODIES bodies of the configuration's
  training-set generator (`scenarios.training_bodies`, cubes and balls of
  20..32 cells, compliance log-U[1e-9, 1e-4], random pinned surface
  vertices; seed 1, so none is the benchmark body), the network trained on
  the GPU on them; then the plain V-cycle PCG on the benchmark body with
  its coarse sweeps replaced by the learned correction, timed like the
  plain leg, beside the same solver with a single coarse Jacobi sweep (the
  cheapest non-learned coarse correction)."""
  from controllable_pbd_3d_gb300 import scenarios
  from controllable_pbd_3d_gb300.learned import (CoarseNet, coarse_energy, collect_pairs,
                                                 train_on_bodies)
  peaks_all = json.load(open(os.path.join(HERE, 'MEASURED_PEAKS.json'))) if os.path.exists(
      os.path.join(HERE, 'MEASURED_PEAKS.json')) else {}
  tc_peak = float(peaks_all.get('bf16_tflops', 1900.0))
  net = CoarseNet(seed=1)
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  losses, data = train_on_bodies(net, scenarios.training_bodies(LEARNED_TRAIN_BODIES, seed=1,
                                                                sides=(20, 32)),
                                 pairs_per_body=32, every=8, steps=1500, batch=8, lr=2e-3)
  torch.cuda.synchronize()
  t_train = time.perf_counter() - t0
  # held-out pairs of the benchmark body: the network's coarse energy beside
  # one Jacobi sweep's and the reference's 50 sweeps'
  xr, x0, t, invm, comp = workload(args.size)
  g, rc = collect_pairs(dict(x_ref=xr, x0=x0, t_i=t, invm=invm, compliance=comp), 32, 8)
  e_net = coarse_energy(g, rc, net.correction(g, rc)).mean().item()
  e_one = coarse_energy(g, rc, ((2.0 / 3.0) * g.diag_inv[None, :] * rc.reshape(-1, g.n))
                        .reshape(rc.shape)).mean().item()
  for _ in range(3):
    net.weights(g)
  t_fwd = _event_time(torch, lambda: net.weights(g), 20)
  fb = net_forward_bytes(g.n, g.nnz)
  flops = 2 * 2 * g.n * 128 * 64  # the two tensor-core layers
  roof = {'kernel': 'coarse network weights pass (k_net_l1 + 2 x k_net_layer: gather + '
                    'mma.sync bf16 tile GEMM + epilogue)', 'bound': 'hbm',
          'achieved': round(fb / t_fwd / 1e9, 1), 'peak': hbm, 'unit': 'GB/s',
          'frac': round(fb / t_fwd / 1e9 / hbm, 4), 'peak_kind': kind,
          'algorithmic_bytes_per_launch': int(fb), 'launch_us': round(t_fwd * 1e6, 2),
          'tensor_tflops': round(flops / t_fwd / 1e12, 3),
          'tensor_frac': round(flops / t_fwd / 1e12 / tc_peak, 5),
          'working_set_note': 'the graph (ah, columns) and the bf16 features stay in L2; '
                              'the neighbour gathers are L2 traffic', 'traffic': None}

  def timed(extra, with_net):
    kw = dict(SOLVER_KW)
    kw.update(PLAIN_KW)
    kw.update(extra)
    sl, _, _ = make_solver(torch, args.size, kw, args.constraints)
    if with_net:
      sl.set_coarse_net(net)
    sl.autotune(reps=5)
    k = max(1, args.plain_steps)
    tl, stl = time_steps(torch, sl, k, 0)
    del sl
    torch.cuda.empty_cache()
    return k, tl, stl

  k, tl, stl = timed(dict(precond='learned'), True)
  k1, t1, st1 = timed(dict(coarse_sweeps=1), False)
  out = {'value': round(k / tl, 4), 'unit': UNIT, 'steps': k,
         'newton_iters_per_step': sum(x['newton_iters'] for x in stl) / k,
         'cg_iters_per_step': sum(x['cg_iters_total'] for x in stl) / k,
         'learned_solves': sum(x['learned_solves'] for x in stl),
         'fallbacks': sum(x['learned_fallbacks'] for x in stl),
         'rejected': sum(x['learned_rejected'] for x in stl),
         'config': 'the plain leg with the coarse sweeps replaced by e_c = w * r_c / diag(A_c), '
                   'w = c sigmoid(y), c = 1.9 / row sums of |Ah|, y from the 3-layer '
                   'message-passing network (hidden 64, bf16 tensor-core layers) on the '
                   'level-1 graph, computed once per Newton iteration; trained off-body',
         'train': {'bodies': LEARNED_TRAIN_BODIES, 'generator': 'scenarios.training_bodies, '
                   'seed 1, sides 20..32', 'pairs': int(sum(r.shape[0] for _, r in data)),
                   'adam_steps': 1500, 'batch': 8, 'seconds': round(t_train, 2),
                   'loss_first20': float(losses[:20].mean()),
                   'loss_last50': float(losses[-50:].mean())},
         'held_out_coarse_energy': {'network': e_net, 'one_jacobi_sweep': e_one},
         'one_sweep_ablation': {'value': round(k1 / t1, 4), 'unit': UNIT, 'steps': k1,
                                'cg_iters_per_step': sum(x['cg_iters_total'] for x in st1) / k1,
                                'config': 'the plain leg with one coarse Jacobi sweep'},
         'roofline': roof}
  out['vs_one_sweep'] = round(out['value'] / out['one_sweep_ablation']['value'], 3)
  return out


def fast_kw(args):
  kw = dict(SOLVER_KW)
  kw.update(FAST_KW)
  if args.no_graph:
    kw['use_graph'] = False
  if args.primal is not None:
    kw['primal'] = bool(args.primal)
  return kw


def plain_leg(torch, args, hbm, kind, constraints):
  """The plain float32 AMG-PCG on the same workload: the reference's
  V-cycle PCG on CSR matrices, each CG solve one CUDA graph with a
  device-side loop, its row-kernel tile shapes picked by the autotuner.
  The length + volume body warms up like the fast leg (3 substeps) and
  times --plain-steps substeps (default 3); every ARAP substep runs the
  full 20 Newton iterations (~25 s), so ARAP times one substep."""
  kwp = dict(SOLVER_KW)
  kwp.update(PLAIN_KW)
  sp_, _, _ = make_solver(torch, args.size, kwp, constraints)
  shapes = sp_.autotune(reps=5)
  warm = 0 if constraints == 'arap' else min(args.warmup, 3)
  for i in range(warm):
    sp_.step(i)
  k_plain = 1 if constraints == 'arap' else max(1, args.plain_steps)
  tp, stp = time_steps(torch, sp_, k_plain, warm)
  roof_csr = roofline_csr(torch, sp_, hbm, kind)
  plain = {'value': round(k_plain / tp, 4), 'unit': UNIT, 'steps': k_plain, 'warmup': warm,
           'newton_iters_per_step': sum(x['newton_iters'] for x in stp) / k_plain,
           'cg_iters_per_step': sum(x['cg_iters_total'] for x in stp) / k_plain,
           'config': 'CSR V-cycle PCG (2-level tet aggregation, 50 coarse Jacobi sweeps, '
                     'smoother weight min(2/3, 4/(3 lambda_max))), each CG solve one CUDA '
                     'graph with a device-side WHILE loop',
           'row_shapes': {str(l): c for l, c in shapes.items()},
           'row_shape_us': {str(l): round(t, 2) for l, (_, t) in sp_.last_tuning.items()},
           'roofline': roof_csr}
  del sp_
  torch.cuda.empty_cache()
  return plain


# the benchmark configuration's mixed-precision multilevel variant of the
# plain solver: 4-5 levels (the tet aggregation, then matrix-graph
# aggregation down to at most 400 rows), float32 smoothing and transfers,
# float64 CG scalars and a float64 dense Cholesky solve of the coarsest level
MIXED_KW = dict(max_levels=3, max_coarse=400, coarse_solver='dense')


def mixed_leg(torch, args, constraints):
  """The plain AMG-PCG with the mixed-precision multilevel hierarchy
  (MIXED_KW), timed like the plain leg."""
  kw = dict(SOLVER_KW)
  kw.update(PLAIN_KW)
  kw.update(MIXED_KW)
  sm, _, _ = make_solver(torch, args.size, kw, constraints)
  sm.autotune(reps=5)
  warm = min(args.warmup, 3)
  for i in range(warm):
    sm.step(i)
  k = max(1, args.plain_steps)
  tm, stm = time_steps(torch, sm, k, warm)
  out = {'value': round(k / tm, 4), 'unit': UNIT, 'steps': k, 'warmup': warm,
         'levels': [int(r) for r in stm[-1]['rows'] if r],
         'newton_iters_per_step': sum(x['newton_iters'] for x in stm) / k,
         'cg_iters_per_step': sum(x['cg_iters_total'] for x in stm) / k,
         'status': stm[-1]['status'],
         'config': 'CSR V-cycle PCG over the tet aggregation plus matrix-graph aggregation '
                   '(aggregates of 8) to <= 400 rows, float32 smoothing and transfers, '
                   'float64 CG scalars, float64 dense Cholesky on the coarsest level; each '
                   'CG solve one CUDA graph'}
  del sm
  torch.cuda.empty_cache()
  return out


def run_ours(args):
  import torch
  ws, rank, local = dist_init(args)
  torch.cuda.set_device(local)
  from controllable_pbd_3d_gb300 import _native as N
  hbm, kind = peaks()
  cons = args.constraints
  kw = fast_kw(args)
  s, x, compliance = make_solver(torch, args.size, kw, cons)
  for i in range(args.warmup):
    s.step(i)
  torch.cuda.synchronize()
  barrier(ws)
  L = N.lib()
  c0 = L.mgpbd_launch_count()
  flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device='cuda')
  with ClockSampler(local) as clk:
    t, st = time_steps(torch, s, args.steps, args.warmup, flush)
  del flush
  launches = L.mgpbd_launch_count() - c0
  barrier(ws)
  t_max = max_over_ranks(ws, t)
  newton = sum(x['newton_iters'] for x in st)
  cg = sum(x['cg_iters_total'] for x in st)
  value = replica_value(ws, args.steps, t_max)

  roof = roofline_from_steps(st, s.n_tets, s.n_verts, FAST_KW['cheb_degree'], hbm, kind,
                             args.size, cons, operator_shape(s))
  roof['matrix_free_apply'] = roofline_matrix_free(torch, s, hbm, kind)
  st0 = st[-1]
  n_verts, n_cons = s.n_verts, s.n_tets
  n_tets = s.n_mesh_tets
  init_s = s.init_s
  del s, x
  torch.cuda.empty_cache()

  # end to end through the public API with host buffers, on a fresh solver
  # over the same substeps as the timed ones (the warm-started solves get
  # cheaper as the body settles, so later substeps would not compare)
  s, x, _ = make_solver(torch, args.size, kw, cons)
  for i in range(args.warmup):
    s.step(i)
  xh = torch.empty_like(x, device='cpu').pin_memory()
  xh.copy_(x)
  vh = torch.empty_like(x, device='cpu').pin_memory()
  vh.copy_(s.v_v)
  torch.cuda.synchronize()
  barrier(ws)
  t0 = time.perf_counter()
  for i in range(args.steps):
    x.copy_(xh, non_blocking=True)
    s.v_v.copy_(vh, non_blocking=True)
    s.step(args.warmup + i)
    xh.copy_(x, non_blocking=True)
    vh.copy_(s.v_v, non_blocking=True)
    torch.cuda.synchronize()
  t_e2e = max_over_ranks(ws, time.perf_counter() - t0)
  e2e = {'value': round(ws * args.steps / t_e2e, 3), 'unit': UNIT,
         'h2d_bytes_per_step': 2 * x.numel() * 4, 'd2h_bytes_per_step': 2 * x.numel() * 4,
         'substeps': f'{args.warmup}..{args.warmup + args.steps - 1} of a fresh solver '
                     '(the timed ones)'}
  del s, x
  torch.cuda.empty_cache()

  plain = None if args.no_plain else plain_leg(torch, args, hbm, kind, cons)
  out = {
      'metric': METRIC, 'value': round(value, 3), 'unit': UNIT, 'n_gpus': ws,
      'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(t_max * 1e3 / args.steps, 3),
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
      'data': 'synthetic (seeded hex-grid cube; reference meshes unavailable)',
      'config': bench_config(args, ws, n_verts, n_tets, n_cons, st0['nnz'][0], compliance),
      'solver': ('FAST: primal warm start + ' if kw.get('primal') else 'FAST: ') +
                f'dual persistent Chebyshev-8 CG on {"D^-1 A" if kw.get("cheb_scale") == "jacobi" else "A"}' +
                (', each substep\'s first solve started from the previous substep\'s solution'
                 if kw.get('warm_substep') else ''),
      'levels': [int(r) for r in st0['rows'] if r],
      'newton_iters_per_step': newton / args.steps, 'cg_iters_per_step': cg / args.steps,
      'cg_iters_per_s': round(ws * cg / t_max, 1), 'gpu_launches': int(launches),
      'clocks': clk.summary(), 'e2e': e2e, 'roofline': roof,
      'init_s': round(init_s, 3),
  }
  if plain is not None:
    out['plain_fp32_amg_pcg'] = plain
    out['speedup_vs_plain'] = round(value / ws / plain['value'], 2)
  if not args.no_mixed and cons == 'edge_volume':
    out['mixed_multilevel_amg_pcg'] = mixed_leg(torch, args, cons)
  if not args.no_batch and ws == 1 and cons == 'edge_volume':
    # the batched configuration, one timed substep after one warm-up
    bl = batch_line(args, 1, 1)
    out['batched'] = {k: bl[k] for k in ('value', 'unit', 'steps', 'warmup', 'ms_per_step',
                                         'newton_iters_per_step', 'cg_iters_per_step',
                                         'status', 'solver', 'roofline', 'clocks',
                                         'gpu_launches')}
    out['batched']['config'] = bl['config']
  if not args.no_learned:
    lrn = learned_leg(torch, args, hbm, kind)
    if plain is not None:
      lrn['speedup_vs_plain'] = round(lrn['value'] / plain['value'], 3)
      lrn['one_sweep_ablation']['speedup_vs_plain'] = round(
          lrn['one_sweep_ablation']['value'] / plain['value'], 3)
    out['learned_amg_pcg'] = lrn
  if cons != 'arap' and not args.no_arap:
    # the reference step's own constraint (one ARAP constraint per tet) on
    # the same body: the fast step and the plain AMG-PCG
    k = max(1, min(args.steps, 5))
    sa, _, _ = make_solver(torch, args.size, kw, 'arap')
    for i in range(min(args.warmup, 3)):
      sa.step(i)
    ta, sta = time_steps(torch, sa, k, args.warmup)
    arap = {'constraints': CONSTRAINT_NAMES['arap'], 'value': round(k / ta, 4), 'unit': UNIT,
            'steps': k, 'newton_iters_per_step': sum(x['newton_iters'] for x in sta) / k,
            'cg_iters_per_step': sum(x['cg_iters_total'] for x in sta) / k,
            'nnz_level0': sta[-1]['nnz'][0],
            'roofline': roofline_from_steps(sta, sa.n_tets, sa.n_verts, FAST_KW['cheb_degree'],
                                            hbm, kind, args.size, 'arap', operator_shape(sa))}
    del sa
    torch.cuda.empty_cache()
    if not args.no_plain:
      arap['plain_fp32_amg_pcg'] = plain_leg(torch, args, hbm, kind, 'arap')
      arap['speedup_vs_plain'] = round(arap['value'] / arap['plain_fp32_amg_pcg']['value'], 2)
    out['arap'] = arap
  if rank == 0 and not args.no_cpu_baseline:
    sub = CpuSubsteps(args.size, cons)
    per, k, newton_c, cg_c = sub.run(1, CPU_BUDGET_S)
    out['cpu_baseline'] = cpu_line(sub, per, k, newton_c, cg_c)
  if rank == 0:
    print(json.dumps(out), flush=True)
  if ws > 1:
    import torch.distributed as dist
    dist.destroy_process_group()


def run_profile_solve(args):
  """One linear solve (substep 0, Newton iteration 0) of the workload, for
  profilers: the persistent kernel (one launch), or with --profile-path
  kernels the per-phase kernels launched from a host loop (no CUDA graph)."""
  import torch
  kw = dict(SOLVER_KW)
  kw.update(FAST_KW if args.profile_precond == 'cheb' else PLAIN_KW)
  kw['use_graph'] = False
  kw['persistent'] = args.profile_path == 'persistent'
  if args.primal is not None:
    kw['primal'] = bool(args.primal)
  kw['maxiter_cg'] = args.profile_maxiter
  s, x, _ = make_solver(torch, args.size, kw, args.constraints)
  s.make_prediction()
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  s._residual_norm_gpu()
  s._fill_A_and_update_gpu()
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  it = s._gpu_solver.solve(s._b_gpu, s._dlam_gpu)
  torch.cuda.synchronize()
  print(json.dumps({'profile_solve': args.profile_precond, 'size': args.size,
                    'constraints': args.constraints, 'cg_iters': it,
                    'seconds': round(time.perf_counter() - t0, 4),
                    'status': s.stats()['status']}), flush=True)


def run_profile_rap(args):
  """The Galerkin coarse level of the length + volume level-0 matrix of a
  `--size`^3 cube, built on the device (`mgpbd_device_galerkin`: copies in,
  the k_rap_* kernels, copies out) and on the host, for profilers and the
  setup figures: one JSON line with both times and whether they agree."""
  import torch
  from controllable_pbd_3d_gb300.tet_aggregation import (galerkin_structure,
                                                         galerkin_structure_device)
  kw = dict(SOLVER_KW)
  kw.update(PLAIN_KW)
  s, x, _ = make_solver(torch, args.size, kw, 'edge_volume')
  g = s._gpu_solver
  A0 = g._gpu_As[0]
  ip = A0.indptr.cpu().numpy()
  ix = A0.indices.cpu().numpy()[:A0.nnz]
  a = A0.data.cpu().numpy()[:A0.nnz]
  agg = g._agg[0].cpu().numpy()
  n_agg = g._gpu_As[1].n_rows
  del s, g
  torch.cuda.empty_cache()
  t0 = time.perf_counter()
  dev = galerkin_structure_device(ip, ix, a, agg, n_agg)
  t_dev = time.perf_counter() - t0
  t0 = time.perf_counter()
  host = galerkin_structure(ip, ix, a, agg, n_agg)
  t_host = time.perf_counter() - t0
  same = all(np.array_equal(u, v) for u, v in zip(host, dev[:4]))
  print(json.dumps({'profile_rap': args.size, 'rows': int(len(ip) - 1), 'nnz': int(A0.nnz),
                    'aggregates': int(n_agg), 'coarse_nnz': int(len(host[1])),
                    'device_s_with_copies': round(t_dev, 4), 'host_s': round(t_host, 4),
                    'bit_identical': bool(same)}), flush=True)


def run_profile_net(args):
  """The coarse network's weights pass on the level-1 graph of a
  `--size`^3 cube (pairs from one plain Newton iteration, 100 Adam steps),
  repeated --profile-reps times, for profilers; one JSON line."""
  import torch
  torch.cuda.set_device(0)
  from controllable_pbd_3d_gb300.learned import CoarseNet
  kwr = dict(SOLVER_KW)
  kwr.update(PLAIN_KW)
  kwr['maxiter'] = 1
  sr, _, _ = make_solver(torch, args.size, kwr, args.constraints)
  sr.record_coarse(64, 8)
  sr.step(0)
  rc, _ = sr.recorded_coarse()
  g = sr.coarse_graph().snapshot()
  net = CoarseNet(seed=1)
  net.fit(g, rc, steps=100, batch=8, lr=2e-3)
  torch.cuda.synchronize()
  for _ in range(args.profile_reps):
    w = net.weights(g)
  torch.cuda.synchronize()
  print(json.dumps({'profile_net': args.size, 'n1': g.n, 'nnz1': g.nnz,
                    'weights_mean': float(w.mean()), 'reps': args.profile_reps}))


SLAB_DIMS = (100, 25, 100)  # the 100 x 100 x 25 slab, y (25) the thin axis
SLAB_COMPLIANCE = 1e-10
SLAB_DRAG = dict(distance=0.5, frames=60)
SUBSTEPS_PER_FRAME = 5


def run_slab(args):
  """The stiff-drag slab: 100 x 100 x 25 hexes (265,226 vertices, 1.25 M
  tets, 5 per hex) with one length constraint per tet edge and one volume
  constraint per tet, compliance 1e-10, one long edge pinned and the
  opposite corner dragged 0.5 along +z over 60 frames as a kinematic
  vertex (moved before each frame of 5 substeps).  The fast step only (the
  plain AMG-PCG is hours at this size); one JSON line with the same
  metric."""
  import torch
  from controllable_pbd_3d_gb300 import _native as N
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from controllable_pbd_3d_gb300.scenarios import DragDriver, drag_slab
  torch.cuda.set_device(0)
  hbm, kind = peaks()
  t_setup = time.perf_counter()
  sl = drag_slab(*SLAB_DIMS)
  x = torch.tensor(sl['x0'], device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(sl['x_ref'], device='cuda'),
                     torch.tensor(sl['invm'], device='cuda'),
                     torch.tensor(sl['t_i'], device='cuda'), None, [0.0, -9.8, 0.0], DT,
                     compliance=SLAB_COMPLIANCE, constraints='edge_volume', **fast_kw(args))
  s.init()
  t_setup = time.perf_counter() - t_setup
  drv = DragDriver(s, sl['drag'], **SLAB_DRAG)

  def substep(i):
    if i % SUBSTEPS_PER_FRAME == 0:
      with torch.no_grad():
        s.v_p[drv.vertex] = drv.target(i // SUBSTEPS_PER_FRAME)
    s.step(i // SUBSTEPS_PER_FRAME)

  for i in range(args.warmup):
    substep(i)
  torch.cuda.synchronize()
  L = N.lib()
  c0 = L.mgpbd_launch_count()
  flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device='cuda')
  stream = torch.cuda.current_stream()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  st = []
  with ClockSampler(0) as clk:
    torch.cuda.synchronize()
    e0.record(stream)
    for i in range(args.warmup, args.warmup + args.steps):
      substep(i)
      st.append(s.stats())
      flush.fill_(i)
    e1.record(stream)
    torch.cuda.synchronize()
  t = e0.elapsed_time(e1) / 1e3
  launches = L.mgpbd_launch_count() - c0
  xs = x.cpu().numpy()
  target = drv.target((args.warmup + args.steps - 1) // SUBSTEPS_PER_FRAME).cpu().numpy()
  roof = roofline_from_steps(st, s.n_tets, s.n_verts, FAST_KW['cheb_degree'], hbm, kind,
                             0, 'edge_volume', operator_shape(s))
  out = {
      'metric': METRIC, 'value': round(args.steps / t, 4), 'unit': UNIT, 'n_gpus': 1,
      'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(t * 1e3 / args.steps, 1),
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
      'data': 'synthetic (hex-grid slab)',
      'config': {'workload': '100x100x25 hex slab, 5 tets/hex, one long edge pinned, the '
                             'opposite corner dragged 0.5 along +z over 60 frames '
                             f'({SUBSTEPS_PER_FRAME} substeps per frame)',
                 'n_verts': s.n_verts, 'n_tets': s.n_mesh_tets,
                 'constraints': CONSTRAINT_NAMES['edge_volume'], 'n_constraints': s.n_tets,
                 'nnz_level0': st[-1]['nnz'][0], 'levels': st[-1]['rows'],
                 'compliance': SLAB_COMPLIANCE, 'dt': DT, 'rel_res_cg': 1e-6,
                 'l2': 'flushed between timed substeps (256 MB write, inside the timed region)',
                 'setup_s': round(t_setup, 1)},
      'solver': 'FAST: dual persistent Chebyshev-8 CG on A',
      'newton_iters_per_step': sum(r['newton_iters'] for r in st) / args.steps,
      'cg_iters_per_step': sum(r['cg_iters_total'] for r in st) / args.steps,
      'max_cg_iters_last_solve': max(r['cg_iters_last'] for r in st),
      'maxiter_cg': SOLVER_KW['maxiter_cg'],
      'gpu_launches': int(launches), 'clocks': clk.summary(), 'roofline': roof,
      'drag_vertex_error': float(np.abs(xs[sl['drag']] - target).max()),
      'pinned_edge_moved': bool(not np.array_equal(xs[sl['pinned']], sl['x0'][sl['pinned']])),
      'finite': bool(np.isfinite(xs).all()), 'status': st[-1]['status']}
  print(json.dumps(out), flush=True)


BATCH_BODIES = 128
SOLVER_BODY_CG = True  # one CG per body (the library default)
BATCH_DIMS = (6, 30)
BATCH_COMPLIANCE = (1e-8, 1e-5)


def batch_line(args, steps, warmup):
  """The batched configuration: 128 independent bodies, hex-grid cells per
  axis uniform in 6..30 (5 tets per hex, cell size 1/40, top face pinned,
  1 % jitter), each with its own compliance log-uniform in [1e-8, 1e-5],
  length + volume constraints, packed into one block-diagonal system.
  The FAST step with per-body Newton loops (own residual, stopping test
  and line-search step per body) and one CG per body in one persistent
  launch, each substep one replay of the captured graph (`--no-graph`: the
  host loop).  Returns the JSON dict (fast step only: the plain AMG-PCG on
  the stiffest of these bodies does not reach 1e-6 within the cap)."""
  import torch
  from controllable_pbd_3d_gb300 import _native as N
  from controllable_pbd_3d_gb300.batch import BodyBatch, random_bodies
  torch.cuda.set_device(0)
  hbm, kind = peaks()
  t_setup = time.perf_counter()
  n_bodies = args.batch_bodies or BATCH_BODIES
  bodies = random_bodies(n_bodies, seed=0, dims=BATCH_DIMS, compliance=BATCH_COMPLIANCE)
  # (no warm substep start here: measured at the batch's second substep it
  # cost 5 % more CG iterations than starting from 0)
  bkw = fast_kw(args)
  bkw['warm_substep'] = False
  batch = BodyBatch(bodies, [0.0, -9.8, 0.0], DT, constraints='edge_volume', **bkw)
  batch.init()
  s = batch.solver
  t_setup = time.perf_counter() - t_setup
  for i in range(warmup):
    batch.step(i)
  torch.cuda.synchronize()
  L = N.lib()
  c0 = L.mgpbd_launch_count()
  flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device='cuda')
  with ClockSampler(0) as clk:
    t, st = time_steps(torch, s, steps, warmup, flush)
  launches = L.mgpbd_launch_count() - c0
  bst = s.body_stats()
  roof = roofline_from_steps(st, s.n_tets, s.n_verts, FAST_KW['cheb_degree'], hbm, kind, 0,
                             'edge_volume', operator_shape(s))
  if SOLVER_BODY_CG:
    roof['kernel'] = 'k_jcg_bodies (one dual persistent Chebyshev-8 CG per body, one launch)'

  comp = np.array([b.compliance for b in bodies])
  out = {
      'metric': METRIC, 'value': round(steps / t, 4), 'unit': UNIT, 'n_gpus': 1,
      'steps': steps, 'warmup': warmup, 'ms_per_step': round(t * 1e3 / steps, 1),
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
      'data': 'synthetic (seeded hex-grid bodies)',
      'config': {'workload': f'{n_bodies} independent bodies, cells per axis uniform in '
                             f'{BATCH_DIMS[0]}..{BATCH_DIMS[1]}, 5 tets/hex, packed block-diagonal',
                 'n_verts': s.n_verts, 'n_tets': batch.n_tets,
                 'constraints': CONSTRAINT_NAMES['edge_volume'], 'n_constraints': s.n_tets,
                 'compliance': f'per body, log-uniform in [{BATCH_COMPLIANCE[0]:g}, '
                               f'{BATCH_COMPLIANCE[1]:g}] (drawn {comp.min():.2e} .. '
                               f'{comp.max():.2e})',
                 'dt': DT, 'rel_res_cg': 1e-6,
                 'l2': 'flushed between timed substeps (256 MB write, inside the timed region)',
                 'setup_s': round(t_setup, 1)},
      'solver': ('FAST, per-body Newton loops, one CG per body in one persistent launch '
                 '(Chebyshev-8 on A)' if SOLVER_BODY_CG else
                 'FAST, per-body Newton loops: one Chebyshev-8 CG on A over the pack, verified '
                 'per body') + (', the substep one captured CUDA graph' if not args.no_graph
                                else ', host loop'),
      'newton_iters_per_step': sum(r['newton_iters'] for r in st) / steps,
      'cg_iters_per_step': sum(r['cg_iters_total'] for r in st) / steps,
      'cg_launches_per_step': sum(r['cg_launches'] for r in st) / steps,
      'body_newton_iters_last_step': {'min': int(bst['newton_iters'].min()),
                                      'median': float(np.median(bst['newton_iters'])),
                                      'max': int(bst['newton_iters'].max())},
      'maxiter_cg': SOLVER_KW['maxiter_cg'], 'status': st[-1]['status'],
      'gpu_launches': int(launches), 'clocks': clk.summary(), 'roofline': roof}
  del batch, s, flush
  torch.cuda.empty_cache()
  return out


def run_batch(args):
  """`--workload batch`: the batched configuration's own JSON line."""
  print(json.dumps(batch_line(args, args.steps, args.warmup)), flush=True)


TRAIN_SET_BODIES = 256  # the training-set configuration
TRAIN_PAIRS, TRAIN_EVERY, TRAIN_STEPS = 4, 8, 4000


def run_train(args):
  """The learned correction's training-set configuration: 256 seeded
  bodies (hex-grid cubes, side uniform in 20..40, half of them projected to
  a ball, compliance log-uniform in [1e-9, 1e-4], 1-4 % of surface vertices
  pinned; `scenarios.training_bodies(256, seed=0)`), TRAIN_PAIRS restricted
  residuals per body from the plain solver's first V-cycles (its CG stopped
  after TRAIN_PAIRS * TRAIN_EVERY + 1 iterations), the 3-layer network
  (hidden 64) trained on the GPU on all of them; then its coarse energy on
  held-out pairs of the benchmark body beside one Jacobi sweep's.  One JSON
  line; nothing here is a timed substep."""
  import torch
  from controllable_pbd_3d_gb300 import scenarios
  from controllable_pbd_3d_gb300.learned import CoarseNet, coarse_energy, collect_pairs
  torch.cuda.set_device(0)
  limit = TRAIN_PAIRS * TRAIN_EVERY + 1
  data, sides, comps = [], [], []
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  for b in scenarios.training_bodies(TRAIN_SET_BODIES, seed=0):
    g, rc = collect_pairs(b, TRAIN_PAIRS, TRAIN_EVERY, cg_limit=limit)
    sides.append(int(b['side']))
    comps.append(float(b['compliance']))
    if rc.shape[0] > 0:
      data.append((g, rc))
  torch.cuda.synchronize()
  t_collect = time.perf_counter() - t0
  net = CoarseNet(seed=1)
  t0 = time.perf_counter()
  losses = net.fit_many(data, steps=TRAIN_STEPS, batch=TRAIN_PAIRS, lr=2e-3)
  torch.cuda.synchronize()
  t_train = time.perf_counter() - t0
  xr, x0, t, invm, comp = workload(args.size)
  g, rc = collect_pairs(dict(x_ref=xr, x0=x0, t_i=t, invm=invm, compliance=comp), 32, 8)
  e_net = coarse_energy(g, rc, net.correction(g, rc)).mean().item()
  e_one = coarse_energy(g, rc, ((2.0 / 3.0) * g.diag_inv[None, :] * rc.reshape(-1, g.n))
                        .reshape(rc.shape)).mean().item()
  out = {'metric': 'learned coarse correction: training set', 'workload': 'train',
         'data': 'synthetic (seeded training bodies)',
         'config': {'bodies': TRAIN_SET_BODIES, 'generator': 'scenarios.training_bodies(256, seed=0)',
                    'sides': [min(sides), max(sides)],
                    'compliance': [min(comps), max(comps)],
                    'pairs_per_body': TRAIN_PAIRS, 'every': TRAIN_EVERY,
                    'network': '3 message-passing layers, hidden 64, bf16 tensor-core layers'},
         'bodies_with_pairs': len(data), 'pairs': int(sum(r.shape[0] for _, r in data)),
         'collect_s': round(t_collect, 1), 'train_s': round(t_train, 1),
         'adam_steps': TRAIN_STEPS, 'loss_first50': float(losses[:50].mean()),
         'loss_last200': float(losses[-200:].mean()),
         'held_out': f'{args.size}^3 benchmark body, 32 pairs',
         'held_out_coarse_energy': {'network': e_net, 'one_jacobi_sweep': e_one},
         'network_over_one_sweep': round(e_net / e_one, 4) if e_one else None}
  del batch, s, flush
  torch.cuda.empty_cache()
  return out


def run_batch(args):
  """`--workload batch`: the batched configuration's own JSON line."""
  print(json.dumps(batch_line(args, args.steps, args.warmup)), flush=True)


def run_reference(args):
  """The reference algorithm on the host cores (the reference itself needs
  Taichi, absent here): whole substeps of the OpenMP CPU port of the plain
  step, from substep 0, as many as fit in CPU_BUDGET_S (at least one; a
  40^3 substep takes about two minutes on 16 Arm cores).  `steps` is the
  number of substeps actually timed, `steps_requested` the --steps asked
  for.  One JSON line on rank 0; other ranks exit."""
  ws = int(os.environ.get('WORLD_SIZE', '1'))
  rank = int(os.environ.get('RANK', '0'))
  if rank != 0:
    return
  sub = CpuSubsteps(args.size, args.constraints)
  per, k, newton_c, cg_c = sub.run(args.steps, CPU_BUDGET_S)
  port = sub.port
  cpu = cpu_line(sub, per, k, newton_c, cg_c)
  value = cpu['value']
  out = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': k,
         'steps_requested': args.steps, 'warmup': 0, 'warmup_requested': args.warmup,
         'ms_per_step': round(per * 1e3, 1), 'higher_is_better': True, 'scaling': 'weak',
         'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded hex-grid cube)',
         'impl': 'reference',
         'config': bench_config(args, ws, port.nv, port.n_mesh_tets, port.nt, port.nnz0,
                                port.compliance),
         'solver': 'plain FP32 AMG-PCG (two-level tet-aggregation V-cycle PCG), OpenMP CPU port',
         'newton_iters_per_step': newton_c, 'cg_iters_per_step': cg_c,
         'cpu_baseline': cpu,
         'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
  print(json.dumps(out), flush=True)


def arg_parser():
  ap = argparse.ArgumentParser()
  ap.add_argument('--gpus', type=int, default=1)
  ap.add_argument('--steps', type=int, default=10)
  ap.add_argument('--warmup', type=int, default=3)
  ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
  ap.add_argument('--size', type=int, default=40)
  ap.add_argument('--no-cpu-baseline', action='store_true')
  ap.add_argument('--no-mixed', action='store_true')
  ap.add_argument('--no-batch', action='store_true')
  ap.add_argument('--no-plain', action='store_true')
  ap.add_argument('--plain-steps', type=int, default=3)
  ap.add_argument('--no-learned', action='store_true')
  ap.add_argument('--no-arap', action='store_true')
  # the constraint construction of the headline workload
  ap.add_argument('--constraints', default='edge_volume', choices=['edge_volume', 'arap'])
  # same kernels launched from a host loop instead of one CUDA graph per
  # CG solve (ncu cannot profile kernels inside conditional graphs)
  ap.add_argument('--no-graph', action='store_true')
  # --workload batch: fewer bodies than the configuration's 128 (the first
  # bodies of the same seeded draw), for profiler captures
  ap.add_argument('--batch-bodies', type=int, default=0)
  ap.add_argument('--profile-solve', action='store_true')
  ap.add_argument('--profile-rap', action='store_true')
  ap.add_argument('--profile-precond', default='cheb', choices=['cheb', 'vcycle'])
  ap.add_argument('--profile-maxiter', type=int, default=6000)
  # 1/0: with / without the primal (Woodbury) warm start of each CG solve
  ap.add_argument('--primal', type=int, default=None, choices=[0, 1])
  # Chebyshev solve as one persistent kernel, or one kernel per phase
  ap.add_argument('--profile-path', default='persistent', choices=['persistent', 'kernels'])
  # the coarse network's weights pass alone (for ncu)
  ap.add_argument('--profile-net', action='store_true')
  ap.add_argument('--profile-reps', type=int, default=5)
  # cube: the 40^3 headline line with its legs; slab: the stiff-drag slab,
  # batch: the 128-body configuration (one line each, fast step only);
  # train: the learned correction's 256-body training set (no timed substeps)
  ap.add_argument('--workload', default='cube', choices=['cube', 'slab', 'batch', 'train'])
  return ap


def main():
  args = arg_parser().parse_args()
  if args.profile_net:
    run_profile_net(args)
  elif args.workload == 'slab' and args.impl == 'ours':
    run_slab(args)
  elif args.workload == 'batch' and args.impl == 'ours':
    run_batch(args)
  elif args.workload == 'train' and args.impl == 'ours':
    run_train(args)
  elif args.profile_solve:
    run_profile_solve(args)
  elif args.profile_rap:
    run_profile_rap(args)
  elif args.impl == 'reference':
    run_reference(args)
  else:
    run_ours(args)


if __name__ == '__main__':
  main()
