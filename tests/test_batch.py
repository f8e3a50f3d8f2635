"""Packing independent bodies into one block-diagonal MGPBD system."""

import numpy as np
import pytest

from controllable_pbd_3d_gb300.batch import pack_bodies, random_bodies


def test_pack_bodies_is_block_diagonal():
  from oracle.mgpbd_oracle import sparsity_pattern
  bodies = random_bodies(4, seed=3, dims=(2, 4))
  xr, x0, invm, t_i, voff, toff = pack_bodies(bodies)
  assert voff[-1] == len(xr) == len(x0) == len(invm)
  assert toff[-1] * 4 == len(t_i)
  t = t_i.reshape(-1, 4)
  for b, body in enumerate(bodies):
    tb = t[toff[b]:toff[b + 1]]
    assert tb.min() >= voff[b] and tb.max() < voff[b + 1]
    np.testing.assert_array_equal(tb - voff[b], body.t_i.reshape(-1, 4))
  # the dual matrix couples tets only within a body
  ip, ix = sparsity_pattern(t_i, len(t))
  body_of = np.searchsorted(toff, np.arange(len(t)), side='right') - 1
  rows = np.repeat(np.arange(len(t)), np.diff(ip))
  np.testing.assert_array_equal(body_of[rows], body_of[ix])


def test_random_bodies_ranges():
  bodies = random_bodies(16, seed=0)
  for b in bodies:
    n = len(b.t_i) // 20  # 5 tets per hex
    assert 6 ** 3 <= n <= 30 ** 3
    assert 1e-8 <= b.compliance <= 1e-5
    assert (b.invm == 0).any() and (b.invm == 1).any()


@pytest.mark.gpu
def test_batched_solve_equals_per_body_solves(cuda):
  """One CG solve of the packed system gives every body the solution of
  its own system (block diagonal), for bodies of different sizes and
  compliances."""
  from controllable_pbd_3d_gb300.batch import BodyBatch
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  g, dt = [0.0, -9.8, 0.0], 1 / 300
  # the dual persistent solve (the primal warm start is for moderate
  # stiffness; these bodies go down to compliance 1e-8)
  kw = dict(mode='fast', precond='cheb', rel_tol_cg=1e-9, tol_cg=1e-14, maxiter_cg=6000,
            primal=False)
  bodies = random_bodies(3, seed=1, dims=(3, 7))

  def first_solve(s):
    s.make_prediction()
    s.lambdaf.zero_()
    s._compute_C_and_gradC()
    s._residual_norm_gpu()
    s._fill_A_and_update_gpu()
    s._gpu_solver.solve(s._b_gpu, s._dlam_gpu)
    return s._dlam_gpu.detach().cpu().numpy().copy()

  batch = BodyBatch(bodies, g, dt, **kw)
  batch.init()
  dl = first_solve(batch.solver)
  for b, body in enumerate(bodies):
    x = cuda.tensor(body.x0, device='cuda')
    s = MGPBDSolverGPU(x, cuda.tensor(body.x_ref, device='cuda'),
                       cuda.tensor(body.invm, device='cuda'), cuda.tensor(body.t_i, device='cuda'),
                       None, g, dt, compliance=body.compliance, **kw)
    s.init()
    ref = first_solve(s)
    got = dl[batch.tet_off[b]:batch.tet_off[b + 1]]
    assert float(np.abs(got - ref).max()) <= 1e-4 * float(np.abs(ref).max()), b


@pytest.mark.gpu
def test_batched_edge_volume_solve_equals_per_body_solves(cuda):
  """The same with one length constraint per edge and one volume constraint
  per tet: each body's constraints (its volume block, then its edges) take
  its own compliance, and the packed solve equals the per-body solves."""
  from controllable_pbd_3d_gb300.batch import BodyBatch
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  g, dt = [0.0, -9.8, 0.0], 1 / 300
  kw = dict(mode='fast', precond='cheb', rel_tol_cg=1e-9, tol_cg=1e-14, maxiter_cg=6000,
            primal=False, constraints='edge_volume')
  bodies = random_bodies(3, seed=4, dims=(3, 6))

  def first_solve(s):
    s.make_prediction()
    s.lambdaf.zero_()
    s._compute_C_and_gradC()
    s._residual_norm_gpu()
    s._fill_A_and_update_gpu()
    s._gpu_solver.solve(s._b_gpu, s._dlam_gpu)
    return s._dlam_gpu.detach().cpu().numpy().copy()

  batch = BodyBatch(bodies, g, dt, **kw)
  batch.init()
  owner = batch.constraint_body()
  nt = batch.n_tets
  alpha = batch.solver.alpha_tilde.cpu().numpy()
  for b, body in enumerate(bodies):
    assert np.allclose(alpha[owner == b], body.compliance / dt ** 2, rtol=1e-6)
  dl = first_solve(batch.solver)
  for b, body in enumerate(bodies):
    x = cuda.tensor(body.x0, device='cuda')
    s = MGPBDSolverGPU(x, cuda.tensor(body.x_ref, device='cuda'),
                       cuda.tensor(body.invm, device='cuda'), cuda.tensor(body.t_i, device='cuda'),
                       None, g, dt, compliance=body.compliance, **kw)
    s.init()
    ref = first_solve(s)
    got = np.concatenate([dl[batch.tet_off[b]:batch.tet_off[b + 1]], dl[nt:][owner[nt:] == b]])
    assert len(got) == len(ref)
    assert float(np.abs(got - ref).max()) <= 1e-4 * float(np.abs(ref).max()), b


def test_set_bodies_validates_its_ranges():
  """mgpbd_set_bodies checks the vertex offsets and the constraint ranges on
  the host (no GPU: the mesh pointers are only stored until init)."""
  import ctypes as C
  from controllable_pbd_3d_gb300 import _native as N
  L = N.lib()
  p = N.default_params()
  p.dt = 1.0 / 300
  h = C.c_void_p()
  N.check(L.mgpbd_create(C.byref(p), C.byref(h)), 'mgpbd_create')
  try:
    fake = C.c_void_p(1 << 20)
    nv, nt = 10, 6
    assert L.mgpbd_set_mesh(h, fake, fake, fake, nv, nt, fake, fake) == 0

    def call(vo, segs):
      vo = np.ascontiguousarray(vo, np.int32)
      sg = np.ascontiguousarray(np.asarray(segs, np.int32).reshape(-1))
      return L.mgpbd_set_bodies(h, len(vo) - 1, vo.ctypes.data, len(sg) // 3, sg.ctypes.data)

    assert call([0, 4, 10], [[0, 2, 0], [2, 6, 1]]) == 0
    assert call([0, 4, 10], [[0, 2, 0], [2, 4, 1], [4, 6, 0]]) == 0  # a body in two ranges
    assert call([0, 4, 9], [[0, 2, 0], [2, 6, 1]]) == -1          # vertices do not end at nv
    assert call([0, 4, 4, 10], [[0, 2, 0], [2, 4, 1], [4, 6, 2]]) == -1  # an empty body
    assert call([0, 4, 10], [[0, 3, 0], [2, 6, 1]]) == -1          # overlapping ranges
    assert call([0, 4, 10], [[0, 2, 0], [2, 5, 1]]) == -1          # not up to nt
    assert call([0, 4, 10], [[0, 2, 0], [2, 6, 2]]) == -1          # body id out of range
    assert call([0, 4, 10], [[0, 6, 0], [6, 6, 1]]) == -1          # an empty range
    assert b'bodies' in L.mgpbd_last_error()
  finally:
    L.mgpbd_destroy(h)


@pytest.mark.gpu
@pytest.mark.parametrize('body_cg,warm', [(True, False), (False, False), (True, True)])
def test_per_body_newton_equals_separate_substeps(cuda, body_cg, warm):
  """Packed bodies with per-body Newton loops (own residual, stopping test
  and line-search step; the shared CG solve verified per body) land where
  each body's own substeps land: positions within 1e-5 relative after three
  substeps, and the same Newton iteration count per body.  The Newton loops
  run to a test with margin on both sides (rtol 3e-3: after one iteration
  r/r0 is ~1e-2, after two it sits at the float32 floor, 1e-5 .. 1e-4), so
  every count is decided far from the threshold; the bodies differ in size
  and compliance, so they end their loops at different iterations.  (ARAP
  bodies are left out: the reference's ARAP step never meets its Newton
  test in 20 iterations, and a trajectory cut off mid-iteration is not a
  stable quantity to compare.)"""
  constraints = 'edge_volume'
  from controllable_pbd_3d_gb300.batch import BodyBatch
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  g, dt = [0.0, -9.8, 0.0], 1 / 300
  kw = dict(mode='fast', precond='cheb', cheb_scale='none', cheb_lo=1e-3, primal=False,
            rel_tol_cg=1e-7, tol_cg=1e-14, maxiter_cg=6000, maxiter=10, atol=1e-9, rtol=3e-3,
            kinematic_pins=True, constraints=constraints, warm_substep=warm)
  bodies = random_bodies(4, seed=2, dims=(3, 7), compliance=(1e-8, 1e-5))
  batch = BodyBatch(bodies, g, dt, body_cg=body_cg, **kw)
  assert batch.per_body
  batch.init()
  singles = []
  for body in bodies:
    x = cuda.tensor(body.x0, device='cuda')
    s = MGPBDSolverGPU(x, cuda.tensor(body.x_ref, device='cuda'),
                       cuda.tensor(body.invm, device='cuda'), cuda.tensor(body.t_i, device='cuda'),
                       None, g, dt, compliance=body.compliance, **kw)
    s.init()
    singles.append((s, x))
  for k in range(3):
    batch.step(k)
    its = batch.solver.body_stats()['newton_iters']
    for b, (s, x) in enumerate(singles):
      s.step(k)
      assert its[b] == s.stats()['newton_iters'], (k, b, its, s.stats()['newton_iters'])
    assert batch.solver.stats()['status'] == 0
  for b, (s, x) in enumerate(singles):
    got = batch.positions(b).cpu().numpy().astype(np.float64)
    ref = x.cpu().numpy().astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), b


@pytest.mark.gpu
@pytest.mark.parametrize('body_cg,warm', [(True, False), (False, False), (True, True)])
def test_captured_substep_equals_host_loop(cuda, body_cg, warm):
  """The packed-body substep as one captured CUDA graph (use_graph: the
  Newton loop a device-side while loop, every decision taken on the device)
  and the same substep driven by the host loop take the same decisions in
  the same arithmetic: positions, per-body Newton counts, residuals, steps
  and the Newton log agree bit for bit over three substeps, and the graph
  replays (one capture, three launches).  Both linear solves: one CG per
  body in one launch (body_cg), and one CG over the pack verified per
  body; and the per-body CG with each substep's first solve started from
  the previous substep's solution (warm_substep)."""
  from controllable_pbd_3d_gb300.batch import BodyBatch
  g, dt = [0.0, -9.8, 0.0], 1 / 300
  kw = dict(mode='fast', precond='cheb', cheb_scale='none', cheb_lo=1e-3, primal=False,
            rel_tol_cg=1e-7, tol_cg=1e-14, maxiter_cg=6000, maxiter=10, atol=1e-9, rtol=3e-3,
            kinematic_pins=True, constraints='edge_volume')
  bodies = random_bodies(5, seed=3, dims=(3, 7), compliance=(1e-8, 1e-5))
  runs = {}
  for graph in (True, False):
    batch = BodyBatch(bodies, g, dt, use_graph=graph, body_cg=body_cg, warm_substep=warm, **kw)
    batch.init()
    hist = []
    for k in range(3):
      batch.step(k)
      st = batch.solver.stats()
      hist.append((batch.x.cpu().numpy().copy(), batch.solver.body_stats(),
                   {key: st[key] for key in ('newton_iters', 'cg_iters_total', 'residual',
                                             'residual0', 'omega_last', 'status')},
                   [tuple(e[1:4]) for e in batch.solver.newton_log()]))
    runs[graph] = hist
  for (xg, bg, sg, lg), (xh, bh, sh, lh) in zip(runs[True], runs[False]):
    np.testing.assert_array_equal(xg, xh)
    for key in bg:
      np.testing.assert_array_equal(bg[key], bh[key])
    assert sg == sh
    assert lg == lh
  assert runs[True][-1][2]['status'] == 0


def _block_system(n_bodies=4, seed=1, dims=(4, 8)):
  """The first Newton system of each of `n_bodies` packed bodies (length +
  volume constraints, float64): the blocks, their right-hand sides."""
  import scipy.sparse as sp
  from oracle import mgpbd_oracle as MO
  from oracle.exact_solve import constraint_jacobian
  As, bs = [], []
  for b in random_bodies(n_bodies, seed=seed, dims=dims, compliance=(1e-8, 1e-5)):
    c, ctype, _, _ = MO.edge_volume_system(b.t_i)
    dm, rest, alpha = MO.rest_shape(b.x_ref, c, 0.0, 1 / 300, np.float64, compliance=b.compliance,
                                    ctype=ctype)
    C, g = MO.constraints(b.x0, c, dm, np.float64, ctype=ctype, rest=rest)
    J = constraint_jacobian(c, g, len(b.x_ref))
    w = np.repeat(np.asarray(b.invm, np.float64), 3)
    As.append((J @ sp.diags(w) @ J.T + sp.diags(np.asarray(alpha, np.float64))).tocsr())
    bs.append(-np.asarray(C, np.float64))
  return As, bs


def test_per_body_cg_restated_in_float64():
  """The per-body CG of packed bodies (`k_jcg_bodies`) restated in float64
  (`oracle.exact_solve.chebyshev_pcg_bodies`): on a block-diagonal pack of
  four bodies each body's solution is its own CG's (same shared polynomial)
  to 1e-7, with its iteration count within 2 % (summation order of the
  packed product aside), every body meets its own bound, and one CG over
  the pack run to the smallest body bound needs over 1.5 x the iterations
  of the slowest body."""
  import scipy.sparse as sp
  import scipy.sparse.linalg as sla
  from oracle.exact_solve import chebyshev_pcg, chebyshev_pcg_bodies
  As, bs = _block_system()
  Ab = sp.block_diag(As).tocsr()
  bb = np.concatenate(bs)
  offs = np.cumsum([0] + [len(b) for b in bs])
  idx = [np.arange(offs[k], offs[k + 1]) for k in range(len(bs))]
  lmax = float(sla.eigsh(Ab, k=1, which='LA', tol=1e-10, return_eigenvectors=False)[0])
  x, its = chebyshev_pcg_bodies(lambda v: Ab @ v, bb, idx, lmax=lmax)
  for k, (A, b) in enumerate(zip(As, bs)):
    xs, it = chebyshev_pcg(lambda v, A=A: A @ v, b, lmax=lmax)
    assert np.abs(x[idx[k]] - xs).max() <= 1e-7 * np.abs(xs).max(), k
    assert abs(its[k] - it) <= 0.02 * it, (k, its[k], it)
    assert np.linalg.norm(b - A @ x[idx[k]]) <= 1.01e-6 * np.linalg.norm(b), k
  bound = min(1e-6 * np.linalg.norm(b) for b in bs)
  _, itc = chebyshev_pcg(lambda v: Ab @ v, bb, lmax=lmax, rel_tol=0.0, tol_abs=bound)
  assert itc > 1.5 * max(its), (itc, its)
