"""bench.py's algorithmic-byte model (the numerator of every roofline
fraction it reports) on the 40^3 cube of both constraint constructions, and
the bookkeeping around its ncu traffic table.  Host only."""

import numpy as np
import pytest

from conftest import ROOT  # noqa: F401  (puts the repository root on sys.path)

import bench as B
from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300.edge_volume import edge_volume_system


@pytest.fixture(scope='module')
def cube40():
  xr, t = meshgen.hex_grid_tets(40, 40, 40)
  _, types, edges, _ = edge_volume_system(t)
  return len(xr), len(t) // 4, types, edges


def test_arap_bytes_per_application_and_iteration(cube40):
  nv, nt, _, _ = cube40
  assert (nv, nt) == (68921, 320000)
  assert B.apply_bytes(nt, nv) == 48836844
  assert B.cg_iteration_bytes(nt, nv, 8) == 454694752
  assert B.primal_iteration_bytes(nt, nv, 8) == 445516144


def test_edge_volume_bytes_per_application_and_iteration(cube40):
  nv, nt_mesh, types, edges = cube40
  nc = len(types)
  n2 = int((types == 1).sum())
  assert (nc, n2, len(edges)) == (718520, 398520, 398520)

  class S:  # the two fields operator_shape reads from a solver
    constraint_types = types
    n_tets = nc

  ne, n2s = B.operator_shape(S)
  assert n2s == n2
  # incidence entries: 4 per volume constraint, 2 per length constraint
  assert ne == 4 * nt_mesh + 2 * n2 == 2077040
  assert B.apply_bytes(nc, nv, ne, n2) == 77530284
  assert B.cg_iteration_bytes(nc, nv, 8, ne, n2) == 763946272
  assert B.primal_iteration_bytes(nc, nv, 8, ne, n2) == 662311024


def test_compact_length_constraints_read_fewer_bytes(cube40):
  """The compact form (gradient float4 + two vertex ids, 24 B) replaces the
  64 B of indices and gradient planes of a 4-slot constraint."""
  nv, nt_mesh, types, _ = cube40
  nc, n2 = len(types), int((types == 1).sum())
  ne = 4 * nt_mesh + 2 * n2
  assert B.apply_bytes(nc, nv, ne, 0) - B.apply_bytes(nc, nv, ne, n2) == 40 * n2
  per_apply_full = B.primal_iteration_bytes(nc, nv, 1, ne, 0)
  per_apply_compact = B.primal_iteration_bytes(nc, nv, 1, ne, n2)
  assert per_apply_full - per_apply_compact == 40 * n2


def test_traffic_table_has_a_source_per_entry():
  assert set(B.TRAFFIC_PER_IT_40) == set(B.TRAFFIC_SOURCE)
  for cons, t in B.TRAFFIC_PER_IT_40.items():
    assert cons in B.CONSTRAINT_NAMES and all(v > 0 for v in t.values())


def test_roofline_from_steps_picks_the_dominant_kernel():
  """Two timed substeps, stats as the library reports them: the kernel with
  more GPU time becomes the headline roofline, the other goes under 'other',
  and the traffic ratio uses the per-launch algorithmic bytes."""
  nv, nt, n2 = 68921, 718520, 398520
  ne = 4 * (nt - n2) + 2 * n2
  st = [dict(ms_warm=7.6, ms_dual=100.0, cg_iters_warm=56, cg_iters_total=770, cg_launches=2,
             newton_iters=1, cg_path='primal')] * 2
  r = B.roofline_from_steps(st, nt, nv, 8, 6701.2, 'measured', 40, 'edge_volume', (ne, n2))
  assert r['kernel'].startswith('k_jcg<0>') and r['other']['kernel'].startswith('k_pcg<0>')
  per_launch = B.cg_iteration_bytes(nt, nv, 8, ne, n2) * 714
  assert r['algorithmic_bytes_per_launch'] == per_launch
  assert r['us_per_cg_iteration'] == pytest.approx(100.0e3 / 714, abs=0.01)
  assert r['achieved'] == pytest.approx(per_launch / 0.1 / 1e9, rel=1e-3)
  # measured DRAM bytes per CG iteration times this launch's iterations
  assert r['traffic'] == int(B.TRAFFIC_PER_IT_40['edge_volume']['k_jcg'] * 714)
  assert r['traffic_over_algorithmic'] == pytest.approx(r['traffic'] / per_launch, abs=1e-4)
  assert r['share_of_cg_gpu_time'] + r['other']['share_of_cg_gpu_time'] == pytest.approx(1, abs=2e-3)
  assert np.isclose(r['frac'], r['achieved'] / 6701.2, atol=1e-4)
  # the DRAM rate over the same launch time, far below the algorithmic one
  assert r['dram_gbs'] == pytest.approx(r['traffic'] / 0.1 / 1e9, rel=1e-3)
  assert r['dram_frac'] < 0.5 * r['frac']


def test_reference_arm_prints_one_contract_line():
  """`bench.py --impl reference` (the OpenMP CPU port of the plain step on
  the host cores) prints one JSON line with the contract's keys: impl,
  cpu_baseline (kind, cores, sample, value = the line's) and an e2e block
  with no host-device copies."""
  import json
  import subprocess
  import sys
  from conftest import ROOT
  out = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--steps', '1',
                        '--warmup', '0', '--size', '10'], cwd=ROOT, capture_output=True, text=True,
                       timeout=600, check=True).stdout.strip().splitlines()
  assert len(out) == 1
  d = json.loads(out[0])
  assert d['impl'] == 'reference' and d['unit'] == 'substeps/s' and d['higher_is_better']
  assert d['value'] > 0 and d['n_gpus'] == 1
  cb = d['cpu_baseline']
  assert cb['value'] == d['value'] and cb['kind'] == 'port' and cb['cores'] >= 1 and cb['sample']
  assert d['e2e'] == {'value': d['value'], 'unit': d['unit'], 'h2d_bytes_per_step': 0,
                      'd2h_bytes_per_step': 0}
  # whole substeps actually timed, the workload described as the GPU arm does
  assert d['steps'] >= 1 and d['steps_requested'] == 1 and cb['cpu_model']
  assert 'whole substep' in cb['sample']
  assert d["cg_iters_per_step"] < 20000  # the CPU port converges (no cap)
  assert set(d["config"]) == {'workload', 'n_verts', 'n_tets', 'constraints', 'n_constraints',
                              'nnz_level0', 'compliance', 'dt', 'rel_res_cg', 'l2',
                              'parallelism'}
  assert d['config']['n_tets'] == 5000 and d['config']['n_constraints'] == 11930


def test_cpu_substeps_load_no_product_library():
  """The CPU legs build their structure with the oracle: libmgpbd.so is
  never mapped into the process."""
  import subprocess
  import sys
  from conftest import ROOT
  code = ('import bench; s = bench.CpuSubsteps(5); s.run(1, 0.0); '
          'print(open("/proc/self/maps").read().count("libmgpbd"))')
  out = subprocess.run([sys.executable, '-c', code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600, check=True).stdout.strip().splitlines()
  assert out[-1] == '0'


def test_bench_defaults_and_legs():
  """The driver's plain `python bench.py` runs the headline with every leg
  (N = 1, 10 timed substeps after 3 warm-up); each leg can be left out."""
  import bench
  a = bench.arg_parser().parse_args([])
  assert (a.gpus, a.steps, a.warmup, a.impl, a.workload, a.size) == (1, 10, 3, 'ours', 'cube', 40)
  assert a.constraints == 'edge_volume'
  assert not (a.no_plain or a.no_mixed or a.no_learned or a.no_arap or a.no_batch or
              a.no_cpu_baseline or a.no_graph)
  b = bench.arg_parser().parse_args(['--workload', 'batch', '--batch-bodies', '16', '--no-graph'])
  assert b.workload == 'batch' and b.batch_bodies == 16 and b.no_graph
  assert bench.FAST_KW['warm_substep'] and bench.FAST_KW['cheb_scale'] == 'none'
  assert bench.MIXED_KW['coarse_solver'] == 'dense' and bench.MIXED_KW['max_levels'] >= 2
