"""The benchmark's own solver at the benchmark's configurations, against the
float64 oracle with exact linear solves.

The solver is `bench.py`'s FAST step exactly (`SOLVER_KW` + `FAST_KW`:
dual persistent CG preconditioned by a Chebyshev-8 polynomial in A, CG to
relative residual 1e-6, each substep's first solve started from the
previous substep's solution, Newton maxiter 20 / atol 1e-4 / rtol 1e-2, no
damping, pinned vertices kinematic) on the length + volume constraint
system.  The oracle
(`oracle/mgpbd_oracle.py`, `linear='exact'`) runs the same Newton loop and
line search in float64 and solves every Newton system to a dual residual of
1e-11 |b| (`oracle/exact_solve.py`); its trajectories are committed
fixtures (`tests/golden/make_headline.py`).

Bar (the benchmark's): positions within 1e-5 relative (max |x_gpu - x_ref|
<= 1e-5 max |x_ref|) after the stated substeps, and the same Newton
iteration count per substep where the oracle's Newton test is not within
1 % of its threshold.

* C1: the 10^3 cube, compliance 1e-6, 100 frames x 5 substeps, checked after
  substeps 1..20 and every 20th.
* C2: the 40^3 cube of the benchmark, two substeps, for the compliance drawn
  by seeds 0 (1.53e-6, the benchmark's draw), 1 (3.6e-7) and 4 (5.2e-5);
  the stiffest draws, seeds 3 (2.7e-9) and 11 (4.4e-9), on the 20^3 cube
  for three substeps (the float64 oracle factorises its vertex system
  there; at 40^3 its iterative route takes hours per substep).  Every CG
  solve of these runs must end below the iteration cap.
* FAST and the plain FP32 AMG-PCG (the CSR V-cycle PCG the benchmark
  compares against) reach the same positions at 40^3.
"""

import os

import numpy as np
import pytest

import bench
from conftest import GOLDEN, golden
from controllable_pbd_3d_gb300 import scenarios
from oracle import mgpbd_oracle as MO

POS_TOL = 1e-5


def headline_kw(**extra):
  kw = dict(bench.SOLVER_KW)
  kw.update(bench.FAST_KW)
  kw.update(extra)
  return kw


def gpu_body(torch, n, seed, compliance=None, kw=None):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xr, x0, t, invm, drawn = scenarios.cube_body(n, seed)
  comp = drawn if compliance is None else compliance
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], bench.DT,
                     compliance=comp, constraints='edge_volume',
                     **(headline_kw() if kw is None else kw))
  s.init()
  return s, x, x0


def newton_counts(z):
  return (~np.isnan(z['newton_residuals'])).sum(axis=1)


def borderline(z, rtol=1e-2, atol=1e-4, margin=0.01):
  """Substeps whose Newton test was within `margin` (relative) of its
  threshold at some iteration: there a last-digit difference may add or
  save a Newton iteration."""
  out = []
  for i, row in enumerate(z['newton_residuals']):
    r = row[~np.isnan(row)]
    thr = max(atol, rtol * r[0])
    if np.any(np.abs(r[1:] - thr) <= margin * thr):
      out.append(i)
  return set(out)


# ----------------------------------------------------------------------------
# CPU: the oracle and its fixtures
# ----------------------------------------------------------------------------


def test_oracle_constraint_set_is_the_products():
  """The oracle's own length + volume builder equals the library's."""
  from controllable_pbd_3d_gb300.edge_volume import edge_volume_system
  _, _, t, _, _ = scenarios.cube_body(7, 3)
  for a, b in zip(MO.edge_volume_system(t), edge_volume_system(t)):
    np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def test_exact_solve_reaches_its_tolerance():
  """Both routes of the exact solve (factorised K, and CG on K) give dual
  residuals below 1e-11 |b| on a stiff (2.7e-9) and a soft (5.2e-5) body."""
  from oracle.exact_solve import ExactDualSolve
  for seed in (3, 4):
    xr, x0, t, invm, comp = scenarios.cube_body(5, seed)
    c, ty, _, _ = MO.edge_volume_system(t)
    dm, rest, al = MO.rest_shape(xr, c, 1e6, bench.DT, np.float64, comp, ty)
    C, g = MO.constraints(x0, c, dm, np.float64, ty, rest)
    for direct_max in (None, 0):
      ex = ExactDualSolve(c, g, invm, al, direct_max=direct_max)
      dlam, rel = ex.solve(-C, 1e-11)
      assert rel <= 1e-11, (seed, direct_max, rel)
      r = -C - ex.apply_A(dlam)
      assert np.linalg.norm(r) <= 1e-11 * np.linalg.norm(C)


def test_c1_fixture_replays():
  """The committed C1 trajectory is the exact oracle's: its first three
  substeps are recomputed here."""
  z = golden('headline_c1.npz')
  xr, x0, t, invm, _ = scenarios.cube_body(10, 0)
  c, ty, _, _ = MO.edge_volume_system(t)
  o = MO.MGPBDOracle(x0, xr, invm, c, [0.0, -9.8, 0.0], bench.DT, dtype=np.float64,
                     compliance=float(z['compliance']), ctype=ty, linear='exact', damp=1.0,
                     maxiter=20, atol=1e-4, rtol=1e-2, kinematic_pins=True)
  o.init()
  for i in range(3):
    o.step(0)
    assert np.abs(o.x - z['x'][i]).max() <= 1e-6
    assert len(o.log) == newton_counts(z)[i]


def test_warm_substep_start_lands_on_the_exact_step():
  """The FAST linear solve restated in float64 with the warm substep start
  (each substep's first solve from the previous substep's first solution,
  `warm_substep`) against the exact-solve oracle over the first substeps of
  C1's body: positions within 1e-7 relative and the same Newton counts
  (borderline tests aside) over 16 substeps, and at least 5 % fewer CG
  iterations than from 0 once the body moves smoothly (substeps 7-16; on
  the first substeps, from rest, the previous solution is a poor guess:
  float64, 1,007 against 1,212 iterations)."""
  z = golden('headline_c1.npz')
  xr, x0, t, invm, _ = scenarios.cube_body(10, 0)
  c, ty, _, _ = MO.edge_volume_system(t)
  common = dict(dtype=np.float64, compliance=float(z['compliance']), ctype=ty, damp=1.0,
                maxiter=20, atol=1e-4, rtol=1e-2, kinematic_pins=True, maxiter_cg=6000,
                tol_cg=1e-12, rel_tol_cg=1e-6)
  warm = MO.MGPBDOracle(x0, xr, invm, c, [0.0, -9.8, 0.0], bench.DT, linear='cheb',
                        warm_substep=True, **common)
  cold = MO.MGPBDOracle(x0, xr, invm, c, [0.0, -9.8, 0.0], bench.DT, linear='cheb', **common)
  warm.init()
  cold.init()
  its_w, its_c = [], []
  skip = borderline(z)
  for i in range(16):
    warm.step(0)
    cold.step(0)
    assert np.abs(warm.x - z['x'][i]).max() <= 1e-7 * np.abs(z['x'][i]).max(), i
    if i not in skip:
      assert len(warm.log) == newton_counts(z)[i], i
    its_w.append(sum(e[2] for e in warm.log))
    its_c.append(sum(e[2] for e in cold.log))
  assert sum(its_w[6:]) <= 0.95 * sum(its_c[6:]), (its_w, its_c)


# ----------------------------------------------------------------------------
# GPU: the benchmark's solver against the fixtures
# ----------------------------------------------------------------------------


@pytest.mark.gpu
def test_c1_full_run_matches_float64_oracle(cuda):
  """C1 in full: 500 substeps, positions within 1e-5 relative of the exact
  float64 oracle at every stored substep, same Newton counts, no CG cap."""
  torch = cuda
  z = golden('headline_c1.npz')
  s, x, _ = gpu_body(torch, 10, 0, compliance=float(z['compliance']))
  want = dict(zip(z['substeps'].tolist(), range(len(z['substeps']))))
  counts = newton_counts(z)
  skip = borderline(z)
  worst = 0.0
  for i in range(500):
    s.step(i // 5)
    st = s.stats()
    assert st['status'] == 0, (i, st['status'])
    if i not in skip:
      # one log row per residual check (the last one ends the loop), as the
      # oracle's Newton log
      assert len(s.newton_log()) == counts[i], i
    if i + 1 in want:
      ref = z['x'][want[i + 1]].astype(np.float64)
      err = float(np.abs(x.cpu().numpy() - ref).max()) / float(np.abs(ref).max())
      worst = max(worst, err)
      assert err <= POS_TOL, (i + 1, err)
  assert worst > 0.0


def cube_fixtures():
  import glob
  import re
  out = []
  for f in sorted(glob.glob(os.path.join(GOLDEN, 'headline_*_seed*.npz'))):
    m = re.match(r'headline_(\d+)_seed(\d+)\.npz', os.path.basename(f))
    if m:
      out.append((int(m.group(1)), int(m.group(2))))
  return out


@pytest.mark.gpu
@pytest.mark.parametrize('n,seed', cube_fixtures())
def test_cube_substeps_match_float64_oracle(cuda, n, seed):
  """The benchmark body (n = 40: 68,921 vertices, 718,520 constraints;
  the stiffest compliance draws on 20^3) with the compliance the seed
  draws: the benchmark's solver within 1e-5 relative of the exact float64
  oracle after every fixture substep."""
  torch = cuda
  z = golden(f'headline_{n}_seed{seed}.npz')
  s, x, x0 = gpu_body(torch, n, seed)
  assert abs(float(z['compliance']) - s.params.compliance) <= 1e-6 * float(z['compliance'])
  for i in range(len(z['disp'])):
    s.step(0)
    assert s.stats()['status'] == 0, (n, seed, i + 1, s.stats())  # no CG cap, no alarm
    ref = x0.astype(np.float64) + z['disp'][i].astype(np.float64)
    err = float(np.abs(x.cpu().numpy() - ref).max()) / float(np.abs(ref).max())
    assert err <= POS_TOL, (n, seed, i + 1, err, s.stats())


@pytest.mark.gpu
def test_fast_and_plain_reach_the_same_positions_at_40(cuda):
  """The benchmark's FAST step and its plain FP32 AMG-PCG denominator (CSR
  V-cycle PCG, one CUDA graph per solve) land within 1e-5 relative of each
  other after two substeps of the 40^3 benchmark body."""
  torch = cuda
  sf, xf, _ = gpu_body(torch, 40, 0)
  sp_, xp, _ = gpu_body(torch, 40, 0, kw={**bench.SOLVER_KW, **bench.PLAIN_KW})
  for i in range(2):
    sf.step(0)
    sp_.step(0)
  a = xf.cpu().numpy().astype(np.float64)
  b = xp.cpu().numpy().astype(np.float64)
  assert np.abs(a - b).max() <= POS_TOL * np.abs(b).max()


def test_the_fast_algorithm_in_float64_is_the_exact_step():
  """The library's FAST linear solve restated in float64 (Chebyshev-8 CG on
  A to relative residual 1e-6, `linear='cheb'`) lands within 1e-8 of the
  exact-solve oracle on the stiffest draw (20^3, compliance 2.7e-9): the
  solve tolerance is not what separates a float32 run from float64 there."""
  z = golden('headline_20_seed3.npz')
  c = golden('headline_20_seed3_cheb.npz')
  _, x0, _, _, _ = scenarios.cube_body(20, 3)
  for i in range(len(z['disp'])):
    a = x0 + z['disp'][i].astype(np.float64)
    b = x0 + c['disp'][i].astype(np.float64)
    assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max(), i


@pytest.mark.gpu
def test_mixed_multilevel_variant_matches_float64_oracle_at_40(cuda):
  """The benchmark configuration's mixed-precision multilevel solver (the
  plain AMG-PCG over 4-5 levels: tet aggregation, then matrix-graph
  aggregation to <= 400 rows, float64 dense Cholesky on the coarsest,
  float64 CG scalars; `bench.MIXED_KW`) on the 40^3 benchmark body: within
  1e-5 relative of the exact float64 oracle after both fixture substeps,
  with no CG cap reached."""
  torch = cuda
  z = golden('headline_40_seed0.npz')
  kw = {**bench.SOLVER_KW, **bench.PLAIN_KW, **bench.MIXED_KW}
  s, x, x0 = gpu_body(torch, 40, 0, kw=kw)
  levels = [int(r) for r in s.stats()['rows'] if r]
  assert 4 <= len(levels) <= 5 and levels[-1] <= 400, levels
  for i in range(len(z['disp'])):
    s.step(0)
    assert s.stats()['status'] == 0, (i + 1, s.stats())
    ref = x0.astype(np.float64) + z['disp'][i].astype(np.float64)
    err = float(np.abs(x.cpu().numpy() - ref).max()) / float(np.abs(ref).max())
    assert err <= POS_TOL, (i + 1, err)
