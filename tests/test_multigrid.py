"""The multigrid pieces around the reference's two-level tet hierarchy.

* Standalone `GPUMultigridSolver(...).setup(A, Ps)` (cons/mgpcg_gpu.py:
  17-30, 175-212, 261-329) on a caller's matrix and aggregation
  prolongations: the Galerkin levels equal the oracle's (pattern bit for
  bit, values to 1e-5), the V-cycle PCG solves to its tolerance, new
  level-0 values refill the coarse levels.
* The mixed-precision options of the benchmark's large configuration: the
  float64 dense Cholesky coarse solve (`coarse_solver='dense'`) and extra
  levels by matrix-graph aggregation (`max_levels`), against the float64
  oracle (`coarse='dense'`, `extra_levels`): V-cycle output to 1e-4
  relative, positions after two substeps to 1e-5 relative; and the dense
  solve's size limit (4,096 coarse rows) as a range error.
"""

import numpy as np
import pytest
import scipy.sparse as sp

from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300.mgpcg_gpu import GPUMultigridSolver
from oracle import mgpbd_oracle as MO


def rel(a, b):
  a = np.asarray(a, np.float64)
  b = np.asarray(b, np.float64)
  return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def arap_body(n, jitter=0.03, seed=1):
  xr, t = meshgen.hex_grid_tets(n, n, n, h=1.0 / n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, h=1.0 / n, jitter=jitter, seed=seed)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  return xr, x0, t, invm


def system(n=6, mu=1e5):
  """A of the reference's first Newton iteration on an n^3 ARAP body (the
  oracle's float32 assembly, diagonal-last rows) and its tet hierarchy."""
  xr, x0, t, invm = arap_body(n)
  nt = len(t) // 4
  dm, _, al = MO.rest_shape(xr, t, mu, 1 / 300, np.float32)
  _, g = MO.constraints(x0, t, dm, np.float32)
  ip, ix = MO.sparsity_pattern(t, nt)
  a = MO.fill_A(ip, ix, t, invm, g, al, np.float32)
  A = sp.csr_matrix((a, ix, ip), shape=(nt, nt))
  aggs, sizes = MO.tet_hierarchy(t, nt)
  Ps = [sp.csr_matrix((np.ones(len(ag)), (np.arange(len(ag)), ag)), shape=(len(ag), nc))
        for ag, nc in zip(aggs, sizes[1:])]
  return A, Ps, aggs, sizes


def test_prolongations_must_be_aggregations():
  """setup's Ps are aggregation operators (one 1 per row); anything else is
  refused before the library is called."""
  A, Ps, aggs, sizes = system(5)
  a, nc = GPUMultigridSolver._aggregates(Ps[0], A.shape[0])
  np.testing.assert_array_equal(a, aggs[0])
  assert nc == sizes[1]
  bad = Ps[0].tolil()
  bad[0, (aggs[0][0] + 1) % sizes[1]] = 1.0  # a row with two entries
  with pytest.raises(ValueError):
    GPUMultigridSolver._aggregates(bad.tocsr(), A.shape[0])
  with pytest.raises(ValueError):
    GPUMultigridSolver._aggregates(Ps[0] * 0.5, A.shape[0])
  with pytest.raises(ValueError):
    GPUMultigridSolver._aggregates(Ps[0], A.shape[0] + 1)


@pytest.mark.gpu
def test_standalone_setup_solve_and_refill(cuda):
  torch = cuda
  A, Ps, aggs, sizes = system(6)
  gm = GPUMultigridSolver(n_smooth=2, omega_jacobi=2.0 / 3.0, maxiter_cg=400,
                          tol_cg=1e-7).setup(A, Ps)
  assert gm.n_levels == 2 and gm._level_sizes == sizes
  # Galerkin level against the oracle's (cons/mgpcg_gpu.py:43-99)
  ci, cx, cidx, coff, _ = MO.galerkin(A.indptr, A.indices, A.data, aggs[0], sizes[1])
  C1 = gm._gpu_As[1]
  np.testing.assert_array_equal(C1.indptr.cpu().numpy(), ci)
  np.testing.assert_array_equal(C1.indices.cpu().numpy()[:len(cx)], cx)
  Ac = (Ps[0].T @ A.astype(np.float64) @ Ps[0]).tocsr()
  Ac.sort_indices()
  assert rel(C1.data.cpu().numpy()[:len(cx)], Ac.data) < 1e-5
  # the V-cycle PCG (absolute tolerance, as the reference)
  rng = np.random.default_rng(0)
  b = rng.standard_normal(A.shape[0]).astype(np.float32)
  x = torch.zeros(A.shape[0], device='cuda')
  it = gm.solve(torch.tensor(b, device='cuda'), x)
  xs = x.cpu().numpy().astype(np.float64)
  assert 0 < it < 400
  assert np.linalg.norm(A.astype(np.float64) @ xs - b) <= 1e-4 * np.linalg.norm(b)
  # new level-0 values (same pattern, still symmetric): 1/diag and the
  # coarse level follow
  s = 1.0 + 0.1 * rng.random(A.shape[0])
  rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
  d2 = (A.data * s[rows] * s[A.indices]).astype(np.float32)  # D A D, same pattern
  A2 = sp.csr_matrix((d2, A.indices, A.indptr), shape=A.shape)
  gm.update_fine_matrix_data(torch.tensor(A2.data, device='cuda'))
  Ac2 = (Ps[0].T @ A2.astype(np.float64) @ Ps[0]).tocsr()
  Ac2.sort_indices()
  assert rel(gm._gpu_As[1].data.cpu().numpy()[:len(cx)], Ac2.data) < 1e-5
  assert rel(gm._gpu_As[0].diag_inv.cpu().numpy(), 1.0 / A2.diagonal()) < 1e-6


@pytest.mark.gpu
def test_standalone_without_prolongations_is_one_level(cuda):
  torch = cuda
  A, _, _, _ = system(3)
  gm = GPUMultigridSolver(maxiter_cg=2000, tol_cg=1e-6).setup(A, [])
  assert gm.n_levels == 1
  b = np.ones(A.shape[0], np.float32)
  x = torch.zeros(A.shape[0], device='cuda')
  gm.solve(torch.tensor(b, device='cuda'), x)
  r = A.astype(np.float64) @ x.cpu().numpy() - b
  assert np.linalg.norm(r) <= 1e-4 * np.linalg.norm(b)


def gpu_arap(torch, xr, x0, t, invm, **kw):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], 1.0 / 300, **kw)
  s.init()
  return s, x


MIXED = {
    'dense-coarse': dict(coarse_solver='dense'),
    'extra-levels': dict(max_levels=2, max_coarse=60),
    'extra-levels-dense': dict(max_levels=2, max_coarse=60, coarse_solver='dense'),
}


@pytest.mark.gpu
@pytest.mark.parametrize('variant', list(MIXED))
def test_mixed_precision_options_match_float64_oracle(cuda, variant):
  torch = cuda
  xr, x0, t, invm = arap_body(7)
  opt = MIXED[variant]
  common = dict(mu=1e5, damp=0.993, maxiter=4, rtol=1e-6, atol=1e-9, maxiter_cg=3000,
                tol_cg=1e-12, rel_tol_cg=1e-7)
  okw = dict(common)
  okw['coarse'] = opt.get('coarse_solver', 'jacobi')
  okw['extra_levels'] = opt.get('max_levels', 0)
  okw['max_coarse'] = opt.get('max_coarse', 400)
  # one V-cycle with the fixed Jacobi weight (the 'safe' weight comes from a
  # power iteration whose estimate differs in its last digits)
  o = MO.MGPBDOracle(x0, xr, invm, t, [0, -9.8, 0], 1 / 300, dtype=np.float64, **okw)
  o.init()
  s, x = gpu_arap(torch, xr, x0, t, invm, **common, **opt)
  g = s._gpu_solver
  assert g.n_levels == len(o.levels)
  for l in range(1, g.n_levels):
    np.testing.assert_array_equal(g._gpu_As[l].indptr.cpu().numpy(), o.levels[l].indptr)
  if 'max_levels' in opt:
    assert g.n_levels >= 3 and g._level_sizes[-1] <= opt['max_coarse']
  s.make_prediction()
  o.make_prediction()
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  s._fill_A_and_update_gpu()
  o.C, o.gradC = MO.constraints(o.x, o.t_i, o.dm_inv, np.float64)
  o.fill_matrices()
  s._residual_norm_gpu()
  b = s._b_gpu.cpu().numpy()
  z = g.vcycle_apply(torch.tensor(b, device='cuda')).cpu().numpy()
  zo = o.vcycle(0, b.astype(np.float64))
  assert rel(z, zo) < 1e-4
  # whole substeps (capped smoother weight: the PCG needs an SPD V-cycle)
  s2, x2 = gpu_arap(torch, xr, x0, t, invm, smoother='safe', **common, **opt)
  o2 = MO.MGPBDOracle(x0, xr, invm, t, [0, -9.8, 0], 1 / 300, dtype=np.float64,
                      smoother='safe', **okw)
  o2.init()
  for k in range(2):
    s2.step(k)
    o2.step(k)
  assert np.abs(x2.cpu().numpy() - o2.x).max() <= 1e-5 * np.abs(o2.x).max()


@pytest.mark.gpu
def test_dense_coarse_solve_limit_is_a_range_error(cuda):
  """The float64 dense coarse factor holds at most 4,096 rows: a coarsest
  level above that (20^3 ARAP body: 9,277 aggregates) is refused at init
  with MGPBD_ERANGE."""
  from controllable_pbd_3d_gb300._native import MGPBDError
  torch = cuda
  xr, x0, t, invm = arap_body(20)
  with pytest.raises(MGPBDError) as e:
    gpu_arap(torch, xr, x0, t, invm, coarse_solver='dense')
  assert e.value.code == -6
  assert 'dense' in str(e.value)
