"""CUDA path (through the C ABI) against the reference's golden vectors and
the oracle.

Tolerances (float32 arithmetic on both sides; the CUDA path uses its own
3x3 SVD and a different summation order than the reference):
  per-stage values   max|gpu - ref| <= 1e-4 * max|ref|   (1e-5 for C)
  positions          max|gpu - ref| <= 1e-5 * max|ref| after the fixture's
                     substeps (the target of the MGPBD step)
Integer structure (pattern, aggregates, coarse pattern, contribution map) is
compared bit for bit.
"""

import numpy as np
import pytest

from conftest import golden, solver_kwargs, step_fixture_names

pytestmark = pytest.mark.gpu

NAMES = step_fixture_names()


def rel(a, b):
  a = np.asarray(a, np.float64)
  b = np.asarray(b, np.float64)
  return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def np_(t):
  return t.detach().cpu().numpy()


def make_solver(torch, z, **extra):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  x = torch.tensor(z['x0'], device='cuda')
  kw = solver_kwargs(z)
  kw.update(extra)
  s = MGPBDSolverGPU(x, torch.tensor(z['x_ref'], device='cuda'),
                     torch.tensor(z['invm'], device='cuda'),
                     torch.tensor(z['t_i'], device='cuda'), None, z['gravity'].tolist(),
                     float(z['dt']), cg_alias=bool(z['cg_alias']), **kw)
  s.init()
  return s, x


@pytest.mark.parametrize('name', NAMES)
def test_init_structure_and_rest_shape(cuda, name):
  z = golden(name)
  s, _ = make_solver(cuda, z)
  g = s._gpu_solver
  np.testing.assert_array_equal(np_(g._gpu_As[0].indices), z['indices'])
  np.testing.assert_array_equal(np_(g._gpu_As[0].indptr), z['indptr'])
  np.testing.assert_array_equal(np_(g._gpu_As[1].indices), z['coarse_indices'])
  np.testing.assert_array_equal(np_(g._gpu_As[1].indptr), z['coarse_indptr'])
  np.testing.assert_array_equal(np_(g._agg[0]), z['agg_ids'])
  assert rel(np_(s.Dm_inv), z['Dm_inv']) < 1e-5
  assert rel(np_(s.alpha_tilde), z['alpha_tilde']) < 1e-5
  assert rel(np_(s.rest_vol), z['rest_vol']) < 1e-5
  assert rel(np_(g._gpu_As[0].data), z['A0_data']) < 1e-4


@pytest.mark.parametrize('name', NAMES)
def test_first_newton_iteration_stages(cuda, name):
  """Each stage of cons/mgpbd_gpu.py:405-440 on identical inputs."""
  z = golden(name)
  s, x = make_solver(cuda, z)
  g = s._gpu_solver
  s.make_prediction()
  assert rel(np_(x), z['it0_x_pred']) < 1e-6
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  assert rel(np_(s.constraints), z['it0_constraints']) < 1e-5
  assert rel(np_(s.gradC), z['it0_gradC']) < 1e-4
  s._fill_A_and_update_gpu()
  assert rel(np_(g._gpu_As[0].data), z['it0_A_data']) < 1e-4
  assert rel(np_(g._gpu_As[1].data), z['it0_coarse_data']) < 1e-4
  assert rel(np_(g._gpu_As[0].diag_inv), z['it0_diag_inv0']) < 1e-4
  assert rel(np_(g._gpu_As[1].diag_inv), z['it0_diag_inv1']) < 1e-4
  s._residual_norm_gpu()
  assert rel(np_(s._b_gpu), z['it0_b']) < 1e-5
  zz = g.vcycle_apply(cuda.tensor(z['it0_b'], device='cuda'))
  assert rel(np_(zz), z['it0_vcycle_z']) < 1e-4
  it = g.solve(s._b_gpu, s._dlam_gpu)
  assert it == int(z['it0_cg_iters'])
  assert rel(np_(s._dlam_gpu), z['it0_dlam']) < 1e-3
  s._scatter_dlam_gpu()
  assert rel(np_(s.dpos), z['it0_dpos']) < 1e-3
  assert rel(np_(s.lambdaf), z['it0_lambda_post']) < 1e-3
  assert s._line_search() == float(z['it0_omega'])


@pytest.mark.parametrize('name', NAMES)
def test_level_spmv_and_jacobi(cuda, name):
  """GPUSparseMatrix.spmv / jacobi_smooth (cons/sparse_gpu.py:123-144) on
  the reference's own first-iteration matrices."""
  z = golden(name)
  s, _ = make_solver(cuda, z)
  g = s._gpu_solver
  s.make_prediction()
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  s._fill_A_and_update_gpu()
  for lvl, A in enumerate(g._gpu_As):
    xv = cuda.tensor(z[f'it0_spmv_x{lvl}'], device='cuda')
    y = cuda.empty_like(xv)
    A.spmv(xv, y)
    assert rel(np_(y), z[f'it0_spmv_y{lvl}']) < 1e-4
    bv = cuda.tensor(z[f'it0_jac_b{lvl}'], device='cuda')
    A.jacobi_smooth(bv, xv, y, s.omega_jacobi)
    assert rel(np_(y), z[f'it0_jac_y{lvl}']) < 1e-4


@pytest.mark.parametrize('name', NAMES)
def test_substep_trajectory(cuda, name):
  """Whole substeps (cons/mgpbd_gpu.py:200-204): positions within 1e-5 of
  the reference's."""
  z = golden(name)
  s, x = make_solver(cuda, z)
  traj = z['x_traj']
  for k in range(len(traj)):
    s.step(k)
    scale = float(np.abs(traj[k]).max())
    err = float(np.abs(np_(x) - traj[k]).max())
    assert err <= 1e-5 * scale, (k, err)
  log = z['newton_log']
  last = s.newton_log()
  assert len(last) == int(np.sum(log[:, 0] == log[-1, 0]))


@pytest.mark.parametrize('mode', ['parity', 'fast'])
def test_cube10_against_float64_oracle(cuda, mode):
  """A 10^3 cube (5000 tets) against the float64 oracle, both run with
  the same options to tight tolerances."""
  from controllable_pbd_3d_gb300 import meshgen
  from oracle.mgpbd_oracle import MGPBDOracle
  n = 10
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=3)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  kw = dict(mu=1e5, damp=0.993, maxiter=6, rtol=1e-6, atol=1e-9, maxiter_cg=200, tol_cg=1e-9,
            rel_tol_cg=1e-7)
  extra = dict(smoother='safe', coarse_solver='jacobi') if mode == 'fast' else {}
  o = MGPBDOracle(x0, xr, invm, t, [0, -9.8, 0], 1 / 300, dtype=np.float64,
                  smoother=extra.get('smoother', 'jacobi'), **kw)
  o.init()
  xt = cuda.tensor(x0, device='cuda')
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  s = MGPBDSolverGPU(xt, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                     cuda.tensor(t, device='cuda'), None, [0, -9.8, 0], 1 / 300, mode=mode, **kw,
                     **extra)
  s.init()
  for k in range(2):
    o.step(k)
    s.step(k)
  err = float(np.abs(np_(xt) - o.x).max())
  assert err <= 1e-5 * float(np.abs(o.x).max()), err


@pytest.mark.parametrize('name', NAMES[:2])
def test_matrix_free_apply_equals_csr(cuda, name):
  """A x from the gradients (no assembly) equals the assembled CSR product
  and the reference's own matrix."""
  z = golden(name)
  s, _ = make_solver(cuda, z)
  s.make_prediction()
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  s._fill_A_and_update_gpu()
  xv = cuda.tensor(z['it0_spmv_x0'], device='cuda')
  y_mf = np_(s.apply_A(xv, matrix_free=True))
  y_csr = np_(s.apply_A(xv, matrix_free=False))
  assert rel(y_mf, y_csr) < 1e-5
  assert rel(y_mf, z['it0_spmv_y0']) < 1e-4
  # the vectorised internal row kernel on both levels
  for lvl in range(2):
    x = cuda.tensor(z[f'it0_spmv_x{lvl}'], device='cuda')
    assert rel(np_(s.level_sweep(lvl, 0, x)), z[f'it0_spmv_y{lvl}']) < 1e-4
    b = cuda.tensor(z[f'it0_jac_b{lvl}'], device='cuda')
    y = s.level_sweep(lvl, 1, x, b, omega=s.omega_jacobi)
    assert rel(np_(y), z[f'it0_jac_y{lvl}']) < 1e-4


# the FAST-mode Chebyshev solve paths: one kernel per phase, the persistent
# kernel on the dual system, the persistent kernel on the primal system
CHEB_PATHS = {'kernels': dict(persistent=False), 'dual': dict(persistent=True, primal=False),
              'primal': dict(persistent=True, primal=True),
              'dual-l2': dict(persistent=2, primal=False), 'primal-l2': dict(persistent=2, primal=True)}


@pytest.mark.parametrize('path', list(CHEB_PATHS))
@pytest.mark.parametrize('degree', [1, 4, 8])
def test_chebyshev_pcg_solves_the_system(cuda, degree, path):
  """The matrix-free Chebyshev-preconditioned CG reaches the requested
  relative residual of the true system (checked in float64 on the host
  with the reference-order CSR matrix)."""
  from controllable_pbd_3d_gb300 import meshgen
  import scipy.sparse as sp
  n = 8
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=4)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xt = cuda.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(xt, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                     cuda.tensor(t, device='cuda'), None, [0, -9.8, 0], 1 / 300, mu=1e5,
                     mode='fast', precond='cheb', cheb_degree=degree, maxiter_cg=3000,
                     tol_cg=1e-12, rel_tol_cg=1e-6, **CHEB_PATHS[path])
  s.init()
  s.make_prediction()
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  s._residual_norm_gpu()
  s._fill_A_and_update_gpu()
  it = s._gpu_solver.solve(s._b_gpu, s._dlam_gpu)
  assert 0 < it < 3000
  # true residual with the float32 CSR values in float64 arithmetic
  g = s._gpu_solver._gpu_As[0]
  s2 = MGPBDSolverGPU(cuda.tensor(np_(xt), device='cuda'), cuda.tensor(xr, device='cuda'),
                      cuda.tensor(invm, device='cuda'), cuda.tensor(t, device='cuda'), None,
                      [0, -9.8, 0], 1 / 300, mu=1e5)
  s2.init()
  s2._compute_C_and_gradC()
  s2._fill_A_and_update_gpu()
  A = s2._gpu_solver._gpu_As[0].to_scipy().astype(np.float64)
  b = np_(s._b_gpu).astype(np.float64)
  xsol = np_(s._dlam_gpu).astype(np.float64)
  rres = np.linalg.norm(b - A @ xsol) / np.linalg.norm(b)
  assert rres < 1e-4, rres
  del g


@pytest.mark.parametrize('path', list(CHEB_PATHS))
def test_fast_cheb_matches_float64_oracle(cuda, path):
  """FAST mode with the matrix-free Chebyshev PCG converges to the same
  positions as the float64 oracle (both solved tightly)."""
  from controllable_pbd_3d_gb300 import meshgen
  from oracle.mgpbd_oracle import MGPBDOracle
  n = 8
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=3)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  kw = dict(mu=1e5, damp=0.993, maxiter=5, rtol=1e-6, atol=1e-9, maxiter_cg=3000, tol_cg=1e-12,
            rel_tol_cg=1e-7)
  o = MGPBDOracle(x0, xr, invm, t, [0, -9.8, 0], 1 / 300, dtype=np.float64, **kw)
  o.init()
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xt = cuda.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(xt, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                     cuda.tensor(t, device='cuda'), None, [0, -9.8, 0], 1 / 300, mode='fast',
                     precond='cheb', **CHEB_PATHS[path], **kw)
  s.init()
  for k in range(2):
    o.step(k)
    s.step(k)
  err = float(np.abs(np_(xt) - o.x).max())
  assert err <= 1e-5 * float(np.abs(o.x).max()), err


@pytest.mark.parametrize('precond', ['cheb', 'vcycle'])
def test_graph_and_host_loops_agree(cuda, precond):
  """The captured device-driven CG and the host-driven launch of the same
  kernels give bit-identical positions."""
  z = golden('step_cube6_mu3e4.npz')
  kw = dict(mode='fast', precond=precond, rel_tol_cg=1e-6, maxiter_cg=2000)
  if precond == 'vcycle':
    kw['smoother'] = 'safe'
  else:
    kw['persistent'] = False  # the per-phase kernels (graph vs host loop)
  s1, x1 = make_solver(cuda, z, use_graph=True, **kw)
  s2, x2 = make_solver(cuda, z, use_graph=False, **kw)
  for k in range(2):
    s1.step(k)
    s2.step(k)
  np.testing.assert_array_equal(np_(x1), np_(x2))
  assert s1.stats()['cg_iters_total'] == s2.stats()['cg_iters_total']


def _block_solver(cuda, n, **kw):
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=5)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  x = cuda.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                     cuda.tensor(t, device='cuda'), None, [0, -9.8, 0], 1 / 300, mu=1e5,
                     damp=0.993, maxiter=2, atol=1e-9, rtol=1e-9, tol_cg=1e-12,
                     rel_tol_cg=1e-5, maxiter_cg=3000, mode='fast', precond='cheb', **kw)
  s.init()
  return s, x


@pytest.mark.parametrize('primal', [False, True])
@pytest.mark.parametrize('n,path', [(36, 'staged'), (44, 'persistent')])
def test_persistent_cg_deterministic_and_matches_per_phase(cuda, n, path, primal):
  """The one-kernel CG (dual or primal system) repeats bit for bit and
  lands where the per-phase kernels (dual system, float64 residual) land:
  on a 36^3 block (233,280 tets) whose per-block operator data is staged in
  shared memory, and on a 44^3 block (425,920 tets) too large to stage,
  where every phase strides over the grid reading from L2."""
  want = {False: path, True: 'primal' if path == 'persistent' else 'primal-staged'}[primal]
  runs = []
  for persistent in (True, True, False):
    s, x = _block_solver(cuda, n, persistent=persistent, primal=primal)
    assert s.stats()['cg_path'] == (want if persistent else 'kernels')
    s.step(0)
    runs.append((np_(x), s.stats()['cg_iters_total'], s.stats()['status']))
  (xa, ia, sa), (xb, ib, sb), (xc, ic, sc) = runs
  np.testing.assert_array_equal(xa, xb)
  assert ia == ib and sa == sb
  assert ia > 0 and (sa & 1) == 0  # no NaN
  if not primal:
    assert abs(ia - ic) <= max(2, ic // 50), (ia, ic)
  scale = float(np.abs(xc).max())
  assert float(np.abs(xa - xc).max()) <= 1e-5 * scale


def test_fast_mode_matches_parity_mode(cuda):
  """The captured device-driven CG computes what the host-driven one does."""
  z = golden('step_cube6_mu3e4.npz')
  s1, x1 = make_solver(cuda, z)
  s2, x2 = make_solver(cuda, z, mode='fast')
  for k in range(2):
    s1.step(k)
    s2.step(k)
  assert float(np.abs(np_(x1) - np_(x2)).max()) <= 1e-6
  assert s1.stats()['cg_iters_total'] == s2.stats()['cg_iters_total']


@pytest.mark.parametrize('path,comp', [('kernels', 2.7e-8), ('dual', 2.7e-8), ('dual', 1.5e-6),
                                       ('primal', 1.5e-6), ('primal', 4.5e-7), ('primal', 1.9e-7),
                                       ('primal', 2.7e-8)])
def test_cheb_solution_matches_direct_solve_on_stiff_body(cuda, path, comp):
  """The first Newton system of a small stiff body (750 tets, cell size
  1/40): the FAST solve's dlam against a float64 sparse direct solve of the
  same system (built from the solver's own b and gradients), to 1e-4.  The
  dual solves hold down to compliance 2.7e-8.  The primal warm start is
  taken where it is accurate (start amplification ~2e5 at 1.5e-6, ~6.5e5 at
  4.5e-7) and declined where its hand-over would leave errors the float32
  dual CG does not remove (~1.5e6 at 1.9e-7, ~1.1e7 at 2.7e-8)."""
  import scipy.sparse as sp
  import scipy.sparse.linalg as spl
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  nx, ny, nz = 5, 5, 6
  xr, t = meshgen.hex_grid_tets(nx, ny, nz, h=1 / 40)
  x0, _ = meshgen.hex_grid_tets(nx, ny, nz, h=1 / 40, jitter=0.01, seed=9)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(nx, ny, nz, axis=1, side='max')] = 0
  dt = 1 / 300
  s = MGPBDSolverGPU(cuda.tensor(x0, device='cuda'), cuda.tensor(xr, device='cuda'),
                     cuda.tensor(invm, device='cuda'), cuda.tensor(t, device='cuda'), None,
                     [0, -9.8, 0], dt, compliance=comp, mode='fast', precond='cheb',
                     rel_tol_cg=1e-9, tol_cg=1e-14, maxiter_cg=6000, **CHEB_PATHS[path])
  s.init()
  s.make_prediction()
  s.lambdaf.zero_()
  s._compute_C_and_gradC()
  s._residual_norm_gpu()
  s._fill_A_and_update_gpu()
  s._gpu_solver.solve(s._b_gpu, s._dlam_gpu)
  b = np_(s._b_gpu).astype(np.float64)
  g = np_(s.gradC).astype(np.float64)
  nt, nv = len(t) // 4, len(xr)
  tt = t.reshape(nt, 4)
  rows = np.repeat(np.arange(nt), 12)
  cols = (3 * tt[:, :, None] + np.arange(3)[None, None, :]).reshape(-1)
  J = sp.csr_matrix((g.reshape(-1), (rows, cols)), shape=(nt, 3 * nv))
  A = (J @ sp.diags(np.repeat(invm.astype(np.float64), 3)) @ J.T +
       sp.diags(np.full(nt, comp / dt / dt))).tocsc()
  exact = spl.spsolve(A, b)
  got = np_(s._dlam_gpu).astype(np.float64)
  err = float(np.abs(got - exact).max() / np.abs(exact).max())
  assert err <= 1e-4, err
  if path == 'primal':
    st = s.stats()
    assert st['warm_declined'] == (1 if comp < 3e-7 else 0), st['warm_amp']


def test_set_hierarchy(cuda):
  """mgpbd_set_hierarchy: the built-in hierarchy passed back in reproduces
  the default solver bit for bit; a different one (pairs of consecutive
  tets) is used as given."""
  from controllable_pbd_3d_gb300 import meshgen
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from oracle.mgpbd_oracle import tet_hierarchy
  n = 6
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.02, seed=4)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, 1)] = 0
  nt = len(t) // 4
  kw = dict(mu=1e5, maxiter=4, maxiter_cg=200, tol_cg=1e-9)

  def make():
    x = cuda.tensor(x0, device='cuda')
    return MGPBDSolverGPU(x, cuda.tensor(xr, device='cuda'), cuda.tensor(invm, device='cuda'),
                          cuda.tensor(t, device='cuda'), None, [0, -9.8, 0], 1 / 300, **kw), x

  s0, x0t = make()
  s0.init()
  aggs, sizes = tet_hierarchy(t, nt)
  s1, x1t = make()
  s1.set_hierarchy(aggs)
  s1.init()
  np.testing.assert_array_equal(np_(s1._gpu_solver._agg[0]), aggs[0])
  for k in range(2):
    s0.step(k)
    s1.step(k)
  np.testing.assert_array_equal(np_(x0t), np_(x1t))
  pairs = np.arange(nt, dtype=np.int32) // 2
  s2, x2t = make()
  s2.set_hierarchy([pairs])
  s2.init()
  np.testing.assert_array_equal(np_(s2._gpu_solver._agg[0]), pairs)
  assert s2.stats()['rows'] == [nt, (nt + 1) // 2]
  s2.step(0)
  assert np.isfinite(np_(x2t)).all()
