"""Generate the golden fixtures by running the reference's own solver code.

Usage (needs a checkout of JamesYang-7/Controllable_PBD_3D; not available on
the GPU machines, which only read the committed `.npz` files):

    python tests/golden/make_golden.py --ref <reference checkout> [--only structure|local|zone|length|adaptive|step]

Taichi is not installed, so `taichi_cpu_shim` stands in for it (see that
module's docstring for what it can and cannot reproduce).  The reference
modules are imported unmodified:

* `cons/tet_aggregation.py` (pure numpy/scipy) gives the aggregation;
* `utils/graph_coloring.py` (pure numpy) gives the tet and vertex
  colourings, and `cons/deform3d.py` (`Deform3D`, driven by
  `cons/framework.py`) and `cons/vbd.py` (`VBDSolver`) give the comparison
  solvers' substeps (`local.npz`);
* `cons/mgpbd_gpu.py` (`MGPBDSolverGPU`) gives the sparsity pattern
  (`_build_sparsity_pattern`), the per-tet precompute, constraint
  gradients, matrix fill, the GPU multigrid setup (`cons/mgpcg_gpu.py`) and
  whole substeps.

One intervention, applied only to the `step` fixtures and to the coarse
structure: scipy's `astype` canonicalises (sorts) CSR indices whenever the
dtype changes.  `GPUMultigridSolver.setup` (`cons/mgpcg_gpu.py:43,104`) calls
`astype`, so the level-0 matrix is uploaded with sorted columns while
`_fill_A_kernel` (`cons/mgpbd_gpu.py:273-324`) keeps writing values in the
diagonal-last order of `_build_sparsity_pattern` (`:153-194`): the fine matrix
is scrambled from the first Newton iteration on.  The fixtures record the
intended semantics (values and columns in the same diagonal-last order) by
making `astype` keep the index order; `asshipped_*` keys record the
unpatched behaviour as evidence.

A second defect sits in the PCG: `vcycle(0)` computes its residual into
`self._r[0]` (`cons/mgpcg_gpu.py:239-240`), which is also the CG residual
vector of `solve` (`:275,303-305`), so every preconditioner application
overwrites the CG residual with `r - A x_presmoothed`.  Each step case is
written twice: `step_<case>.npz` with the V-cycle's level-0 residual kept
apart from the CG residual (the intended algorithm; the wrapper saves and
restores `_r[0]` around `vcycle(0)`), and `step_<case>_cgalias.npz` with the
reference's PCG exactly as shipped.
"""

from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

from controllable_pbd_3d_gb300 import meshgen  # noqa: E402


def sha(*arrays):
  h = hashlib.sha256()
  for a in arrays:
    h.update(np.ascontiguousarray(np.asarray(a, dtype=np.int64)).tobytes())
  return h.hexdigest()


# ----------------------------------------------------------------------------
# loading the reference under the shim
# ----------------------------------------------------------------------------

_ORIG_ASTYPE = None


def load_reference(ref):
  import taichi_cpu_shim
  taichi_cpu_shim.install()
  sys.path.insert(0, ref)
  import cons.mgpbd_gpu as mg  # noqa: F401
  import cons.tet_aggregation as ta  # noqa: F401
  return sys.modules['cons.mgpbd_gpu'], sys.modules['cons.tet_aggregation']


def set_astype_keeps_order(on: bool):
  """Toggle scipy's canonicalise-on-astype (see module docstring)."""
  import scipy.sparse._data as d
  global _ORIG_ASTYPE
  if _ORIG_ASTYPE is None:
    _ORIG_ASTYPE = d._data_matrix.astype

  def astype_keep_order(self, dtype, casting='unsafe', copy=True):
    dtype = np.dtype(dtype)
    if self.dtype != dtype:
      return self._with_data(self.data.astype(dtype, casting=casting, copy=True), copy=True)
    return self.copy() if copy else self

  d._data_matrix.astype = astype_keep_order if on else _ORIG_ASTYPE


# ----------------------------------------------------------------------------
# cases
# ----------------------------------------------------------------------------


def grid_case(nx, ny, nz, jitter, seed, ball=False):
  """Rest shape = regular grid (optionally ball-projected); start = jittered."""
  xr, t = meshgen.hex_grid_tets(nx, ny, nz)
  x0, _ = meshgen.hex_grid_tets(nx, ny, nz, jitter=jitter, seed=seed)
  if ball:
    xr = meshgen.ball_project(xr)
    x0 = meshgen.ball_project(x0)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(nx, ny, nz, axis=1, side='max')] = 0.0
  return xr, x0, t, invm


def asset_case(ref, rel, fixed):
  v, t, _ = meshgen.parse_medit_mesh(os.path.join(ref, 'assets', rel))
  invm = meshgen.lumped_inverse_mass(v, t)
  invm[np.asarray(fixed, np.int64)] = 0.0
  return v, v.copy(), t, invm


STRUCTURE_CASES = {
    # name: (builder, full_coarse) ; full_coarse -> also coarse pattern + map
    'box5x4x5': (lambda ref: grid_case(5, 4, 5, 0.01, 1), True),
    'cube6': (lambda ref: grid_case(6, 6, 6, 0.01, 0), True),
    'box12x3x7': (lambda ref: grid_case(12, 3, 7, 0.01, 3), True),
    'ball8': (lambda ref: grid_case(8, 8, 8, 0.01, 2, ball=True), False),
    'cube10': (lambda ref: grid_case(10, 10, 10, 0.01, 0), False),
    'cube20': (lambda ref: grid_case(20, 20, 20, 0.01, 0), False),
    'simple_sphere': (lambda ref: asset_case(ref, 'simple_sphere/simple_sphere.mesh', [0, 11]), False),
    'spot': (lambda ref: asset_case(ref, 'spot/spot.mesh', [0]), False),
    'cube_tet': (lambda ref: asset_case(ref, 'cube_tet/cube_tet.mesh', [0]), False),
}


class _Rec:
  """SolverBenchmark-shaped recorder (`utils/bench.py:24-55`)."""

  def __init__(self):
    self.frames = []

  def begin_frame(self, f):
    self.frames.append([])

  def record_iteration(self, ite, r, cg_iters=0, omega=1.0):
    self.frames[-1].append((ite, float(r), int(cg_iters), float(omega)))

  def end_frame(self):
    pass


def make_solver(mg, ti, xr, x0, t, invm, **kw):
  n = len(xr)
  v_p = ti.Vector.field(3, dtype=ti.f32, shape=n)
  v_p.from_numpy(x0)
  v_p_ref = ti.Vector.field(3, dtype=ti.f32, shape=n)
  v_p_ref.from_numpy(xr)
  v_invm = ti.field(ti.f32, n)
  v_invm.from_numpy(invm)
  t_i = ti.field(ti.i32, len(t))
  t_i.from_numpy(t)
  t_m = ti.field(ti.f32, len(t) // 4)
  g = kw.pop('gravity', (0.0, -9.8, 0.0))
  dt = kw.pop('dt', 1.0 / 300.0)
  s = mg.MGPBDSolverGPU(v_p, v_p_ref, v_invm, t_i, t_m, ti.Vector(list(g)), dt, **kw)
  return s


def csr_of(m):
  return m.indptr.to_numpy(), m.indices.to_numpy(), m.data.to_numpy()


def structure_fixtures(ref, mg, ta, out):
  import taichi as ti
  res = {}
  for name, (build, full) in STRUCTURE_CASES.items():
    t0 = time.time()
    xr, x0, t, invm = build(ref)
    nt = len(t) // 4
    res[f'{name}/t_i_sha'] = np.array(sha(t))
    res[f'{name}/x_ref'] = xr
    res[f'{name}/t_i'] = t
    # level-0 pattern through the reference method
    s = make_solver(mg, ti, xr, x0, t, invm, mu=1e5)
    s._build_sparsity_pattern()
    res[f'{name}/nnz'] = np.array(s._nnz)
    res[f'{name}/pattern_sha'] = np.array(sha(s._A_indptr, s._A_indices))
    if nt <= 2000:
      res[f'{name}/indptr'] = s._A_indptr
      res[f'{name}/indices'] = s._A_indices
    # hierarchy through the reference module
    Ps, sizes = ta.build_tet_hierarchy(t.copy(), xr.copy(), nt)
    res[f'{name}/sizes'] = np.array(sizes, np.int64)
    if Ps:
      res[f'{name}/agg_ids'] = Ps[0].indices.astype(np.int32)
      adj = ta.build_tet_face_adjacency(t, nt)
      res[f'{name}/adj_deg'] = np.array([len(adj[i]) for i in range(nt)], np.int32)
    if full and Ps:
      set_astype_keeps_order(True)
      s2 = make_solver(mg, ti, xr, x0, t, invm, mu=1e5)
      s2.init()
      gs = s2._gpu_solver
      res[f'{name}/A0_data'] = s2._A_data.copy()
      ip, ix, _ = csr_of(gs._gpu_As[1])
      res[f'{name}/coarse_indptr'] = ip
      res[f'{name}/coarse_indices'] = ix
      res[f'{name}/contrib_fine_idx'] = gs._contrib_maps[0]['fine_idx']
      res[f'{name}/contrib_offsets'] = gs._contrib_offsets[0]
      set_astype_keeps_order(False)
    print(f'[structure] {name}: nt={nt} sizes={sizes} ({time.time() - t0:.1f}s)', flush=True)
  np.savez_compressed(os.path.join(out, 'structure.npz'), **res)


STEP_CASES = {
    # name: (builder, solver kwargs, substeps)
    'box5x4x5_mu1e5': (lambda ref: grid_case(5, 4, 5, 0.01, 1),
                       dict(mu=1e5, damp=0.993), 3),
    'box5x4x5_ls': (lambda ref: grid_case(5, 4, 5, 0.3, 7),
                    dict(mu=1e5, damp=0.993, maxiter=4), 1),
    'cube6_mu3e4': (lambda ref: grid_case(6, 6, 6, 0.02, 5),
                    dict(mu=3e4, damp=0.993, maxiter=3), 1),
}


def step_fixture(ref, mg, name, build, kw, substeps, out, cg_alias):
  import taichi as ti
  t0 = time.time()
  xr, x0, t, invm = build(ref)
  res = {'x_ref': xr, 'x0': x0, 't_i': t, 'invm': invm,
         'gravity': np.array([0.0, -9.8, 0.0], np.float32), 'dt': np.array(1.0 / 300.0)}
  for k, v in kw.items():
    res['param_' + k] = np.array(v)

  # as-shipped evidence: level-0 columns after setup vs. the fill order
  set_astype_keeps_order(False)
  s_bad = make_solver(mg, ti, xr, x0, t, invm, **kw)
  s_bad.init()
  res['asshipped_level0_indices_match'] = np.array(
      np.array_equal(s_bad._gpu_solver._gpu_As[0].indices.to_numpy(), s_bad._A_indices))

  set_astype_keeps_order(True)
  rec = _Rec()
  s = make_solver(mg, ti, xr, x0, t, invm, benchmark=rec, **kw)
  s.init()
  gs = s._gpu_solver
  res['cg_alias'] = np.array(bool(cg_alias))
  if not cg_alias:
    orig_vcycle = gs.vcycle

    def vcycle_keep_r0(level=0):
      saved = gs._r[0].to_numpy() if level == 0 else None
      orig_vcycle(level)
      if level == 0:
        gs._r[0].from_numpy(saved)

    gs.vcycle = vcycle_keep_r0
  res['Dm_inv'] = s.Dm_inv.to_numpy()
  res['rest_vol'] = s.rest_vol.to_numpy()
  res['alpha_tilde'] = s.alpha_tilde.to_numpy()
  res['A0_data'] = s._A_data.copy()
  res['indptr'] = s._A_indptr
  res['indices'] = s._A_indices
  res['agg_ids'] = s._amg_Ps[0].indices.astype(np.int32) if s._amg_Ps else np.zeros(0, np.int32)
  ip, ix, dd = csr_of(gs._gpu_As[1])
  res['coarse_indptr'], res['coarse_indices'], res['coarse_data0'] = ip, ix, dd
  res['contrib_fine_idx'] = gs._contrib_maps[0]['fine_idx']
  res['contrib_offsets'] = gs._contrib_offsets[0]

  # --- first Newton iteration of substep 0, captured around reference calls
  snap = {}
  orig_cg = gs.solve
  orig_ls = s._line_search
  orig_fill = s._fill_A_and_update_gpu

  def fill():
    orig_fill()
    if 'A_data' not in snap:
      snap['constraints'] = s.constraints.to_numpy()
      snap['gradC'] = s.gradC.to_numpy()
      snap['lambda_pre'] = s.lambdaf.to_numpy()
      snap['x_pred'] = s.v_p.to_numpy()
      snap['A_data'] = gs._gpu_As[0].data.to_numpy()
      snap['diag_inv0'] = gs._gpu_As[0].diag_inv.to_numpy()
      snap['coarse_data'] = gs._gpu_As[1].data.to_numpy()
      snap['diag_inv1'] = gs._gpu_As[1].diag_inv.to_numpy()

  def cg(b, x):
    first = 'b' not in snap
    if first:
      snap['b'] = b.to_numpy()
      # one V-cycle on r = b from zero, through the reference's vcycle
      n = gs._level_sizes[0]
      gs._b[0].from_numpy(b.to_numpy())
      gs._x[0].fill(0.0)
      r_saved = gs._r[0].to_numpy()
      gs.vcycle(0)
      gs._r[0].from_numpy(r_saved)
      snap['vcycle_z'] = gs._x[0].to_numpy()
      # level SpMV / Jacobi with a seeded vector
      rng = np.random.default_rng(11)
      for lvl, A in enumerate(gs._gpu_As):
        xv = ti.field(ti.f32, A.n_rows)
        xv.from_numpy(rng.standard_normal(A.n_rows).astype(np.float32))
        yv = ti.field(ti.f32, A.n_rows)
        A.spmv(xv, yv)
        snap[f'spmv_x{lvl}'] = xv.to_numpy()
        snap[f'spmv_y{lvl}'] = yv.to_numpy()
        bv = ti.field(ti.f32, A.n_rows)
        bv.from_numpy(rng.standard_normal(A.n_rows).astype(np.float32))
        A.jacobi_smooth(bv, xv, yv, gs.omega_jacobi)
        snap[f'jac_b{lvl}'] = bv.to_numpy()
        snap[f'jac_y{lvl}'] = yv.to_numpy()
      del n
    it = orig_cg(b, x)
    if first:
      snap['dlam'] = x.to_numpy()
      snap['cg_iters'] = np.array(it)
    return it

  def ls():
    om = orig_ls()
    if 'omega' not in snap:
      snap['dpos'] = s.dpos.to_numpy()
      snap['lambda_post'] = s.lambdaf.to_numpy()
      snap['omega'] = np.array(om)
    return om

  gs.solve = cg
  s._line_search = ls
  s._fill_A_and_update_gpu = fill
  traj = []
  for k in range(substeps):
    s.step(k)
    traj.append(s.v_p.to_numpy())
    if k == 0:
      snap['x_after_substep0'] = s.v_p.to_numpy()
  for k, v in snap.items():
    res['it0_' + k] = v
  res['x_traj'] = np.stack(traj)
  res['v_final'] = s.v_v.to_numpy()
  res['lambda_final'] = s.lambdaf.to_numpy()
  recs = [(f, *r) for f, fr in enumerate(rec.frames) for r in fr]
  res['newton_log'] = np.array(recs, np.float64).reshape(-1, 5)
  set_astype_keeps_order(False)
  suffix = '_cgalias' if cg_alias else ''
  np.savez_compressed(os.path.join(out, f'step_{name}{suffix}.npz'), **res)
  print(f'[step] {name}{suffix}: {len(recs)} newton iterations ({time.time() - t0:.1f}s)', flush=True)


# ----------------------------------------------------------------------------
# comparison solvers: Deform3D (cons/deform3d.py), VBDSolver (cons/vbd.py)
# and the greedy colourings (utils/graph_coloring.py)
# ----------------------------------------------------------------------------

COLOR_CASES = ('box5x4x5', 'cube6', 'box12x3x7', 'simple_sphere', 'spot', 'cube_tet')


def lumped_case(xr, x0, t, pinned):
  """The reference's mass model (utils/geom3d.py:48-59, data/tet_data.py:39-44):
  vertex mass = sum of |vol| / 4, invm = 1 / mass (pinned -> 0), t_m = |vol|."""
  import utils.geom3d as g3
  _, vm, tm = g3.compute_vertex_mass(np.asarray(xr, np.float64), np.asarray(t, np.int64))
  invm = (1.0 / vm).astype(np.float32)
  invm[np.asarray(pinned, np.int64)] = 0.0
  return xr, x0, t, invm, tm.astype(np.float32)


def box_lumped(nx, ny, nz, jitter, seed):
  xr, x0, t, _ = grid_case(nx, ny, nz, jitter, seed)
  return lumped_case(xr, x0, t, meshgen.grid_face_vertices(nx, ny, nz, axis=1, side='max'))


def sphere_lumped(ref, jitter, seed):
  v, t, _ = meshgen.parse_medit_mesh(os.path.join(ref, 'assets/simple_sphere/simple_sphere.mesh'))
  rng = np.random.default_rng(seed)
  x0 = (v + rng.uniform(-jitter, jitter, v.shape)).astype(np.float32)
  return lumped_case(v.astype(np.float32), x0, t, [0, 11])


def disjoint_tets(n, jitter, seed):
  """n separate unit-ish tets (no shared vertex): the parallel default
  method of Deform3D then has no races and equals the serial order."""
  rng = np.random.default_rng(seed)
  base = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0, 0, 0.1]], np.float64)
  xr = np.concatenate([base + [0.3 * k, 0, 0] for k in range(n)]).astype(np.float32)
  x0 = (xr + rng.uniform(-jitter, jitter, xr.shape)).astype(np.float32)
  t = np.arange(4 * n, dtype=np.int32)
  return lumped_case(xr, x0, t, [0])


LOCAL_CASES = {
    # name: (builder, solver, solver kwargs, substeps, passes per substep, gravity)
    'xpbd_gs_box': (lambda ref: box_lumped(4, 3, 4, 0.05, 11), 'xpbd',
                    dict(hydro_alpha=1e-5, devia_alpha=1e-4, method='gauss_seidel'), 2, 10,
                    (0.0, -9.8, 0.0)),
    'xpbd_color_box': (lambda ref: box_lumped(4, 3, 4, 0.05, 11), 'xpbd',
                       dict(hydro_alpha=1e-5, devia_alpha=1e-4, method='graph_coloring'), 2, 10,
                       (0.0, -9.8, 0.0)),
    'xpbd_gs_sphere': (lambda ref: sphere_lumped(ref, 0.02, 3), 'xpbd',
                       dict(hydro_alpha=0.0, devia_alpha=1e-4, method='gauss_seidel'), 2, 10,
                       (0.0, 0.0, 0.0)),
    'xpbd_default_disjoint': (lambda ref: disjoint_tets(24, 0.01, 5), 'xpbd',
                              dict(hydro_alpha=1e-6, devia_alpha=1e-4, method='default'), 2, 6,
                              (0.0, -9.8, 0.0)),
    'vbd_serial_box': (lambda ref: box_lumped(4, 3, 4, 0.05, 11), 'vbd',
                       dict(youngs_modulus=1e4, poissons_ratio=0.3, n_iterations=10,
                            method='serial'), 2, 0, (0.0, -9.8, 0.0)),
    'vbd_color_box': (lambda ref: box_lumped(4, 3, 4, 0.05, 11), 'vbd',
                      dict(youngs_modulus=1e4, poissons_ratio=0.3, n_iterations=10,
                           method='color'), 2, 0, (0.0, -9.8, 0.0)),
    'vbd_color_cheb_box': (lambda ref: box_lumped(4, 3, 4, 0.05, 11), 'vbd',
                           dict(youngs_modulus=1e4, poissons_ratio=0.3, n_iterations=8,
                                rho=0.7, damping=0.05, method='color'), 2, 0, (0.0, -9.8, 0.0)),
    'vbd_serial_sphere': (lambda ref: sphere_lumped(ref, 0.02, 3), 'vbd',
                          dict(youngs_modulus=1e6, poissons_ratio=0.3, n_iterations=50,
                               method='serial'), 1, 0, (0.0, 0.0, 0.0)),
}

LOCAL_DT = 1.0 / 300.0
LOCAL_DAMP = 0.993


def local_fixtures(ref, out):
  import taichi as ti
  from utils import graph_coloring as gc
  import cons.deform3d as d3
  import cons.vbd as vbd
  from cons import framework
  res = {}
  for name in COLOR_CASES:
    t0 = time.time()
    xr, _, t, _ = (STRUCTURE_CASES[name][0])(ref)
    nt, nv = len(t) // 4, len(xr)
    ce = gc.color_elements(t, nt, 4, nv)
    cv = gc.color_vertices(t, nt, 4, nv)
    res[f'color/{name}/t_i'] = np.asarray(t, np.int32)
    res[f'color/{name}/nv'] = np.array(nv)
    res[f'color/{name}/elem_ordered'] = ce.ordered_indices
    res[f'color/{name}/elem_offsets'] = np.asarray(ce.color_offsets, np.int32)
    res[f'color/{name}/vert_ordered'] = cv.ordered_indices
    res[f'color/{name}/vert_offsets'] = np.asarray(cv.color_offsets, np.int32)
    print(f'[color] {name}: {ce.num_colors} tet colours, {cv.num_colors} vertex colours '
          f'({time.time() - t0:.1f}s)', flush=True)
  for name, (build, kind, kw, substeps, passes, g) in LOCAL_CASES.items():
    t0 = time.time()
    xr, x0, t, invm, tm = build(ref)
    n, nt = len(xr), len(t) // 4
    v_p = ti.Vector.field(3, dtype=ti.f32, shape=n)
    v_p.from_numpy(x0)
    v_p_ref = ti.Vector.field(3, dtype=ti.f32, shape=n)
    v_p_ref.from_numpy(xr)
    v_invm = ti.field(ti.f32, n)
    v_invm.from_numpy(invm)
    t_i = ti.field(ti.i32, len(t))
    t_i.from_numpy(t)
    t_m = ti.field(ti.f32, nt)
    t_m.from_numpy(tm)
    case = {'x_ref': xr, 'x0': x0, 't_i': np.asarray(t, np.int32), 'invm': invm, 't_m': tm,
            'gravity': np.array(g, np.float32), 'dt': np.array(LOCAL_DT),
            'damp': np.array(LOCAL_DAMP), 'substeps': np.array(substeps),
            'passes': np.array(passes)}
    traj = []
    if kind == 'xpbd':
      cons = d3.Deform3D(v_p, v_p_ref, v_invm, t_i, t_m, LOCAL_DT, **kw)
      pbd = framework.pbd_framework(v_p, ti.Vector(list(g)), LOCAL_DT, LOCAL_DAMP)
      pbd.add_cons(cons, 0)
      pbd.init_rest_status(0)
      for _ in range(substeps):
        pbd.step(passes)
        traj.append(v_p.to_numpy())
      case['hydro_lambda'] = cons.hydro_lambda.to_numpy()
      case['devia_lambda'] = cons.devia_lambda.to_numpy()
      case['v_final'] = pbd.v_v.to_numpy()
    else:
      s = vbd.VBDSolver(v_p, v_p_ref, v_invm, t_i, t_m, ti.Vector(list(g)), LOCAL_DT,
                        damp=LOCAL_DAMP, **kw)
      s.init()
      case['dm_inv'] = s.Dm_inv.to_numpy()
      case['rest_vol'] = s.rest_vol.to_numpy()
      case['adj_offsets'] = s.vert_adj_offsets.to_numpy()
      case['adj_tets'] = s.vert_tet_adj.to_numpy()
      case['adj_local'] = s.vert_local_id.to_numpy()
      for k in range(substeps):
        s.step(k)
        traj.append(v_p.to_numpy())
      case['v_final'] = s.v_v.to_numpy()
      case['mu_lam'] = np.array([s.mu, s.lam])
    case['x_traj'] = np.stack(traj)
    for k, v in kw.items():
      case['kw_' + k] = np.array(v)
    for k, v in case.items():
      res[f'{name}/{k}'] = v
    print(f'[local] {name}: nv={n} nt={nt} ({time.time() - t0:.1f}s)', flush=True)
  np.savez_compressed(os.path.join(out, 'local.npz'), **res)


def zone_fixtures(ref, out):
  """The reference's AdaptiveZone (cons/adaptive_zone.py) on a seeded body
  whose vertices moved: proximity flags, two face rings around them, and
  strain-rate flags, as int32 per tet."""
  import taichi as ti
  import cons.adaptive_zone as az
  res = {}
  for name, n, seed in (('cube5', 5, 11), ('box6x3x4', None, 12)):
    if n is not None:
      xr, t = meshgen.hex_grid_tets(n, n, n)
    else:
      xr, t = meshgen.hex_grid_tets(6, 3, 4)
    rng = np.random.default_rng(seed)
    x_old = (xr + rng.uniform(-0.02, 0.02, xr.shape)).astype(np.float32)
    x = (x_old + rng.normal(0.0, 0.004, xr.shape)).astype(np.float32)
    nt = len(t) // 4
    v_p = ti.Vector.field(3, dtype=ti.f32, shape=len(x))
    v_p.from_numpy(x)
    v_old = ti.Vector.field(3, dtype=ti.f32, shape=len(x))
    v_old.from_numpy(x_old)
    t_i = ti.field(ti.i32, len(t))
    t_i.from_numpy(t.astype(np.int32))
    zone = az.AdaptiveZone(nt, t_i, v_p)
    center = x.mean(axis=0).astype(np.float32)
    radius = np.float32(0.3)
    zone.update_by_proximity(float(center[0]), float(center[1]), float(center[2]), float(radius))
    prox = zone.tet_active.to_numpy().astype(np.int32).copy()
    zone.expand_zone(2)
    ring2 = zone.tet_active.to_numpy().astype(np.int32).copy()
    threshold, dt = np.float32(3.0), np.float32(1.0 / 300.0)
    zone.update_by_strain(v_old, float(threshold), float(dt))
    strain = zone.tet_active.to_numpy().astype(np.int32).copy()
    res.update({f'{name}_x': x, f'{name}_x_old': x_old, f'{name}_t': t.astype(np.int32),
                f'{name}_center': center, f'{name}_radius': radius,
                f'{name}_threshold': threshold, f'{name}_dt': dt,
                f'{name}_prox': prox, f'{name}_ring2': ring2, f'{name}_strain': strain})
    print(f'[zone] {name}: nt={nt} prox={prox.sum()} ring2={ring2.sum()} strain={strain.sum()}',
          flush=True)
  np.savez_compressed(os.path.join(out, 'zone.npz'), **res)


def length_fixtures(ref, out):
  """One Gauss-Seidel sweep of the reference's LengthCons (cons/length.py)
  over the unique edges of a seeded jittered body: the positions and
  multipliers after the sweep."""
  import taichi as ti
  import cons.length as lc
  from controllable_pbd_3d_gb300.edge_volume import tet_edges
  xr, t = meshgen.hex_grid_tets(3, 2, 2)
  x0, _ = meshgen.hex_grid_tets(3, 2, 2, jitter=0.15, seed=21)
  edges, _ = tet_edges(t)
  rest = np.sqrt(((xr[edges[:, 0]].astype(np.float64) - xr[edges[:, 1]]) ** 2).sum(1))
  invm = np.ones(len(xr), np.float32)
  invm[:3] = 0.0
  compliance, dt = 1e-4, 1.0 / 300.0
  v_p = ti.Vector.field(3, dtype=ti.f32, shape=len(x0))
  v_p.from_numpy(x0.astype(np.float32))
  v_ref = ti.Vector.field(3, dtype=ti.f32, shape=len(xr))
  v_ref.from_numpy(xr.astype(np.float32))
  e_i = ti.field(ti.i32, 2 * len(edges))
  e_i.from_numpy(edges.reshape(-1).astype(np.int32))
  e_rl = ti.field(ti.f32, len(edges))
  e_rl.from_numpy(rest.astype(np.float32))
  v_invm = ti.field(ti.f32, len(xr))
  v_invm.from_numpy(invm)
  cons = lc.LengthCons(v_p, v_ref, e_i, e_rl, v_invm, dt, alpha=compliance,
                       method='gauss_seidel')
  cons.preupdate_cons()
  cons.update_cons()
  np.savez_compressed(os.path.join(out, 'length.npz'), x0=x0.astype(np.float32), edges=edges,
                      rest=rest.astype(np.float32), invm=invm, compliance=compliance, dt=dt,
                      x1=v_p.to_numpy(), lam=cons.lambdaf.to_numpy())
  print(f'[length] {len(edges)} edges', flush=True)


def adaptive_fixture(ref, mg, out):
  """Two substeps of the reference's MGPBDAdaptiveSolver
  (cons/mgpbd_adaptive.py) around its MGPBDSolverGPU, with a tool near one
  corner: the positions and the active flags after each substep (level-0
  order kept, V-cycle residual kept apart, as in the step fixtures)."""
  import taichi as ti
  import cons.adaptive_zone as az
  import cons.mgpbd_adaptive as ma
  xr, x0, t, invm = grid_case(5, 4, 5, 0.02, 3)
  kw = dict(mu=1e5, damp=0.993, maxiter=3)
  tool, radius = (0.9, 0.1, 0.85), 0.45
  set_astype_keeps_order(True)
  s = make_solver(mg, ti, xr, x0, t, invm, **kw)
  s.init()
  gs = s._gpu_solver
  orig_vcycle = gs.vcycle

  def vcycle_keep_r0(level=0):
    saved = gs._r[0].to_numpy() if level == 0 else None
    orig_vcycle(level)
    if level == 0:
      gs._r[0].from_numpy(saved)

  gs.vcycle = vcycle_keep_r0
  zone = az.AdaptiveZone(s.n_tets, s.t_i, s.v_p)
  ad = ma.MGPBDAdaptiveSolver(s, zone)
  traj, masks = [], []
  for k in range(2):
    ad.step(k, tool_pos=tool, tool_radius=radius)
    traj.append(s.v_p.to_numpy())
    masks.append(zone.tet_active.to_numpy().astype(np.int32))
  set_astype_keeps_order(False)
  res = {'x_ref': xr, 'x0': x0, 't_i': t, 'invm': invm,
         'gravity': np.array([0.0, -9.8, 0.0], np.float32), 'dt': np.array(1.0 / 300.0),
         'tool': np.array(tool, np.float32), 'radius': np.array(radius, np.float32),
         'x_traj': np.stack(traj), 'masks': np.stack(masks),
         'alpha_tilde': s.alpha_tilde.to_numpy(), 'cg_alias': np.array(False)}
  for k, v in kw.items():
    res['param_' + k] = np.array(v)
  np.savez_compressed(os.path.join(out, 'adaptive.npz'), **res)
  print(f'[adaptive] active per substep {[int(m.sum()) for m in masks]} of {s.n_tets}',
        flush=True)


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument('--ref', default=os.environ.get('REFERENCE_ROOT'),
                  help='the reference checkout (default: $REFERENCE_ROOT)')
  ap.add_argument('--only', default=None)
  ap.add_argument('--out', default=HERE)
  a = ap.parse_args()
  if not a.ref:
    ap.error('pass --ref <reference checkout> or set REFERENCE_ROOT')
  mg, ta = load_reference(a.ref)
  if a.only in (None, 'structure'):
    structure_fixtures(a.ref, mg, ta, a.out)
  if a.only in (None, 'local'):
    local_fixtures(a.ref, a.out)
  if a.only in (None, 'zone'):
    zone_fixtures(a.ref, a.out)
  if a.only in (None, 'length'):
    length_fixtures(a.ref, a.out)
  if a.only in (None, 'adaptive'):
    adaptive_fixture(a.ref, mg, a.out)
  if a.only in (None, 'step'):
    for name, (build, kw, n) in STEP_CASES.items():
      for alias in (False, True):
        step_fixture(a.ref, mg, name, build, kw, n, a.out, alias)


if __name__ == '__main__':
  main()
