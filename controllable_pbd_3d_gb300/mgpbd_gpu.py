"""`MGPBDSolverGPU` with the constructor, fields and methods of the
reference's `cons/mgpbd_gpu.py:20-446`, running on libmgpbd.so.

Inputs are CUDA tensors (or arrays, copied to the GPU): `v_p` (NV,3) float32
is mutated in place like the reference's Taichi field; `v_p_ref`, `v_invm`,
`t_i` (4*NT int32) and `t_m` are read.  After `init()` the solver-owned
fields (`lambdaf`, `constraints`, `gradC`, `alpha_tilde`, `Dm_inv`,
`rest_vol`, `v_p_old`, `v_predict`, `dpos`, `_b_gpu`, `_dlam_gpu`) are torch
views of the library's device memory; they stay valid while the solver
lives.  Nothing here computes the step on the CPU: if libmgpbd.so cannot be
loaded, construction raises.
"""

from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _native as N

_MODES = {'parity': N.MGPBD_MODE_PARITY, 'fast': N.MGPBD_MODE_FAST}
_COARSE = {'jacobi': N.MGPBD_COARSE_JACOBI, 'dense': N.MGPBD_COARSE_DENSE_F64}
_SMOOTH = {'jacobi': N.MGPBD_SMOOTH_JACOBI, 'safe': N.MGPBD_SMOOTH_JACOBI_SAFE}


class _DeviceArray:
  """Minimal `__cuda_array_interface__` holder used to view library memory."""

  def __init__(self, ptr, shape, typestr):
    self.__cuda_array_interface__ = {
        'shape': tuple(shape), 'typestr': typestr, 'data': (int(ptr), False), 'version': 3,
        'strides': None,
    }


def device_view(ptr, shape, dtype=torch.float32):
  typestr = {torch.float32: '<f4', torch.int32: '<i4', torch.float64: '<f8'}[dtype]
  if int(np.prod(shape)) == 0:
    return torch.empty(shape, dtype=dtype, device='cuda')
  return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device='cuda')


def _cuda(a, dtype, shape=None):
  if isinstance(a, torch.Tensor):
    t = a
    if t.device.type != 'cuda' or t.dtype != dtype or not t.is_contiguous():
      t = t.to(device='cuda', dtype=dtype).contiguous()
  else:
    if hasattr(a, 'to_numpy'):
      a = a.to_numpy()
    t = torch.as_tensor(np.ascontiguousarray(np.asarray(a)), dtype=dtype).cuda()
  if shape is not None:
    t = t.reshape(shape)
  return t


class _Scalar:
  """Stands in for the reference's 0-d Taichi field (`self.damp[None]`)."""

  def __init__(self, v):
    self.v = float(v)

  def __getitem__(self, key):
    return self.v

  def __setitem__(self, key, val):
    raise AttributeError('damp is fixed at construction')


class MGPBDSolverGPU:
  """Multigrid-accelerated global XPBD step (cons/mgpbd_gpu.py:20-446).

  Extra keyword options select the CUDA library's variants:
    mode='parity'  reference algorithm with host-checked loops (default);
    mode='fast'    device-driven CG in one CUDA graph per solve;
    rel_tol_cg     CG also stops at |r| < rel_tol_cg * |b| (0: reference);
    smoother       'jacobi' (omega_jacobi) or 'safe' (omega <= 4/(3 lambda_max));
    coarse_solver  'jacobi' (min(50,n) sweeps) or 'dense' (float64 Cholesky);
    max_levels     extra levels by matrix-graph aggregation (0: reference);
    kinematic_pins vertices with invm == 0 skip the prediction;
    cg_alias       reproduce the reference PCG whose V-cycle overwrites the
                   CG residual (cons/mgpcg_gpu.py:239-240 vs :275);
    compliance     > 0: alpha~ = compliance / dt^2 for every tet;
    precond        'vcycle' (reference) or 'cheb' (FAST only: Chebyshev
                   polynomial of degree cheb_degree on [lmax*cheb_lo, lmax],
                   matrix-free operator, no CSR assembly; cheb_scale
                   'jacobi' builds it on D^-1 A, 'none' on A itself) or
                   'learned' (the
                   V-cycle with its coarse sweeps replaced by the linear
                   correction w * r / diag(A_c), w from a trained CoarseNet
                   attached with set_coarse_net; the plain V-cycle judges it
                   on each solve's first V-cycle -- threshold learned_accept,
                   see include/mgpbd.h -- and takes over on stalls);
    use_graph      FAST: one CUDA graph with a device-side loop per CG solve
                   (False: the same kernels from a host loop); with packed
                   bodies, one graph per substep;
    body_cg        packed bodies: one CG per body in one launch (True) or one
                   CG over the pack, verified per body (False);
    warm_substep   FAST dual persistent CG, one body: start each substep's
                   first solve from the previous substep's solution;
    constraints    'arap' (the reference: one ARAP constraint per tet) or
                   'edge_volume' (one length constraint per unique tet edge
                   and one volume constraint det F - 1 per tet, alpha~ =
                   compliance / dt^2; n_tets then counts constraints, the
                   mesh's tets are in mesh_t_i / n_mesh_tets);
    persistent     FAST + 'cheb': each CG solve is one cooperative persistent
                   kernel (False: one kernel per phase, per use_graph; 2: the
                   persistent kernel reading the operator from L2 instead of
                   staging it in shared memory);
    primal         FAST + 'cheb' + persistent: warm-start each solve through
                   the vertex-space system K y = J^T alpha~^-1 b (Woodbury)
                   to a dual residual of primal_tol |b|, then CG on A;
  """

  def __init__(self, v_p, v_p_ref, v_invm, t_i, t_m, gravity, dt, mu=1e6, damp=1.0, maxiter=20,
               atol=1e-4, rtol=1e-2, maxiter_cg=100, tol_cg=1e-5, n_smooth=2,
               omega_jacobi=2.0 / 3.0, setup_interval=10000, use_line_search=True,
               aggregation='tet', benchmark=None, *, mode='parity', rel_tol_cg=0.0,
               coarse_solver='jacobi', smoother='jacobi', max_levels=0, max_coarse=400,
               kinematic_pins=False, coarse_sweeps=0, cg_alias=False, compliance=0.0,
               precond='vcycle', cheb_degree=8, cheb_lo=0.01, cheb_scale='jacobi',
               use_graph=True, body_cg=True, warm_substep=False,
               persistent=True, primal=False, primal_tol=1e-2, learned_accept=0.1, learned_stall=1000,
               constraints='arap', check_finite=True):
    if aggregation != 'tet':
      raise NotImplementedError(
          "aggregation='pyamg' needs PyAMG's smoothed-aggregation setup, which this "
          "library does not provide; use aggregation='tet'")
    self._lib = N.lib()
    self.v_p = _cuda(v_p, torch.float32, (-1, 3))
    if isinstance(v_p, torch.Tensor) and self.v_p.data_ptr() != v_p.data_ptr():
      raise ValueError('v_p must be a contiguous float32 CUDA tensor (it is updated in place)')
    self.v_p_ref = _cuda(v_p_ref, torch.float32, (-1, 3))
    self.v_invm = _cuda(v_invm, torch.float32, (-1,))
    self.t_i = _cuda(t_i, torch.int32, (-1,))
    self.t_m = t_m
    self.n_verts = self.v_p.shape[0]
    self.n_tets = self.t_i.shape[0] // 4
    if self.v_p_ref.shape[0] != self.n_verts or self.v_invm.shape[0] != self.n_verts:
      raise ValueError('v_p, v_p_ref and v_invm must have the same number of vertices')
    if self.t_i.shape[0] != 4 * self.n_tets:
      raise ValueError('t_i must hold 4 indices per tet')
    # the constraint set: one ARAP constraint per tet (the reference's), or
    # one volume constraint per tet plus one length constraint per edge
    if constraints not in ('arap', 'edge_volume'):
      raise ValueError("constraints must be 'arap' or 'edge_volume'")
    self.constraint_kind = constraints
    self.mesh_t_i = self.t_i
    self.n_mesh_tets = self.n_tets
    self.constraint_types = None
    agg0 = None
    if constraints == 'edge_volume':
      if not compliance > 0:
        raise ValueError("constraints='edge_volume' takes alpha~ = compliance / dt^2: "
                         'pass compliance > 0')
      from .edge_volume import edge_volume_hierarchy, edge_volume_system
      t_host = self.t_i.cpu().numpy()
      c_i, types, self.edges, _ = edge_volume_system(t_host)
      self.constraint_types = types
      self.t_i = torch.tensor(c_i, device=self.v_p.device)
      self.n_tets = len(types)  # constraints (the fields below have this length)
      agg0 = edge_volume_hierarchy(t_host, max_coarse=int(max_coarse))
    self.gravity = [float(g) for g in (gravity.to_numpy() if hasattr(gravity, 'to_numpy') else gravity)]
    self.dt = float(dt)
    self.mu = float(mu)
    self.maxiter = maxiter
    self.atol = atol
    self.rtol = rtol
    self.maxiter_cg = maxiter_cg
    self.tol_cg = tol_cg
    self.n_smooth = n_smooth
    self.omega_jacobi = omega_jacobi
    self.setup_interval = setup_interval
    self.use_line_search = use_line_search
    self.aggregation = aggregation
    self.benchmark = benchmark
    self.damp = _Scalar(damp)
    self.check_finite = check_finite
    self.v_v = torch.zeros_like(self.v_p)

    p = N.default_params()
    p.dt = self.dt
    p.mu = self.mu
    p.damp = float(damp)
    for k in range(3):
      p.gravity[k] = self.gravity[k]
    p.maxiter = int(maxiter)
    p.atol = float(atol)
    p.rtol = float(rtol)
    p.maxiter_cg = int(maxiter_cg)
    p.tol_cg = float(tol_cg)
    p.n_smooth = int(n_smooth)
    p.omega_jacobi = float(omega_jacobi)
    p.setup_interval = int(setup_interval)
    p.use_line_search = int(bool(use_line_search))
    p.mode = _MODES[mode]
    p.rel_tol_cg = float(rel_tol_cg)
    p.coarse_solver = _COARSE[coarse_solver]
    p.smoother = _SMOOTH[smoother]
    p.max_levels = int(max_levels)
    p.max_coarse = int(max_coarse)
    p.kinematic_pins = int(bool(kinematic_pins))
    p.coarse_sweeps = int(coarse_sweeps)
    p.cg_alias = int(bool(cg_alias))
    p.compliance = float(compliance)
    p.precond = {'vcycle': 0, 'cheb': 1, 'learned': 2}[precond]
    p.cheb_degree = int(cheb_degree)
    p.cheb_lo = float(cheb_lo)
    p.cheb_scale = {'jacobi': 0, 'none': 1}[cheb_scale]
    p.use_graph = int(bool(use_graph))
    p.body_cg = int(bool(body_cg))
    p.warm_substep = int(bool(warm_substep))
    p.persistent = int(persistent)  # True / 1, 2 (unstaged) or False / 0
    p.primal = int(bool(primal))
    p.primal_tol = float(primal_tol)
    p.learned_accept = float(learned_accept)
    p.learned_stall = int(learned_stall)
    self.params = p
    h = C.c_void_p()
    N.check(self._lib.mgpbd_create(C.byref(p), C.byref(h)), 'mgpbd_create')
    self._h = h
    N.check(self._lib.mgpbd_set_mesh(h, self.v_p_ref.data_ptr(), self.v_invm.data_ptr(),
                                     self.t_i.data_ptr(), self.n_verts, self.n_tets,
                                     self.v_p.data_ptr(), self.v_v.data_ptr()), 'mgpbd_set_mesh')
    if self.constraint_types is not None:
      N.check(self._lib.mgpbd_set_constraint_types(h, self.constraint_types.ctypes.data),
              'mgpbd_set_constraint_types')
      if agg0 is not None:
        self.set_hierarchy([agg0])
    self._inited = False
    self._gpu_solver = None

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        self._lib.mgpbd_destroy(h)
      except Exception:
        pass
      self._h = None

  # ------------------------------------------------------------------ #
  def _stream(self):
    N.check(self._lib.mgpbd_set_stream(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)),
            'mgpbd_set_stream')

  def _field(self, name, shape):
    ptr = C.c_void_p()
    cnt = C.c_int64()
    N.check(self._lib.mgpbd_field(self._h, N.FIELD[name], C.byref(ptr), C.byref(cnt)), 'mgpbd_field')
    return device_view(ptr.value, shape)

  # cons/mgpbd_gpu.py:92-114
  def set_hierarchy(self, aggs):
    """Use the aggregation hierarchy `aggs` (a list of per-level aggregate
    id arrays: aggs[l] maps level-l rows to level-(l+1) rows) instead of
    the built-in tet aggregation at the next init()."""
    sizes = [self.n_tets]
    for a in aggs:
      a = np.asarray(a)
      if len(a) != sizes[-1]:
        raise ValueError('aggs[l] must have one id per level-l row')
      sizes.append(int(a.max()) + 1 if len(a) else 0)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(a, np.int32) for a in aggs]))
    sz = np.asarray(sizes, np.int32)
    N.check(self._lib.mgpbd_set_hierarchy(self._h, flat.ctypes.data, len(sizes), sz.ctypes.data),
            'mgpbd_set_hierarchy')
    self._inited = False

  def set_bodies(self, vert_off, segments):
    """Independent bodies packed in this mesh, each with its own Newton loop
    (residual, stopping test, line-search step) over a shared, per-body
    verified block-diagonal CG solve.  vert_off: (n_bodies + 1,) vertex
    offsets; segments: (k, 3) rows (begin, end, body) of constraint ranges
    covering all constraints in order.  Before init(); FAST Chebyshev only."""
    vo = np.ascontiguousarray(vert_off, np.int32)
    sg = np.ascontiguousarray(np.asarray(segments, np.int32).reshape(-1, 3))
    N.check(self._lib.mgpbd_set_bodies(self._h, len(vo) - 1, vo.ctypes.data, len(sg),
                                       sg.ctypes.data), 'mgpbd_set_bodies')
    self.n_bodies = len(vo) - 1
    self._inited = False

  def body_stats(self) -> dict:
    """Per body: Newton iterations, first / last residual, last step."""
    n = self.n_bodies
    it = np.zeros(n, np.int32)
    r0, r, om = np.zeros(n), np.zeros(n), np.zeros(n)
    N.check(self._lib.mgpbd_body_stats(self._h, n, it.ctypes.data, r0.ctypes.data, r.ctypes.data,
                                       om.ctypes.data), 'mgpbd_body_stats')
    return {'newton_iters': it, 'residual0': r0, 'residual': r, 'omega': om}

  def init(self):
    self._stream()
    N.check(self._lib.mgpbd_init(self._h), 'mgpbd_init')
    nt, nv = self.n_tets, self.n_verts
    self.lambdaf = self._field('lambdaf', (nt,))
    self.constraints = self._field('constraints', (nt,))
    self.gradC = self._field('gradC', (nt, 4, 3))
    self.alpha_tilde = self._field('alpha_tilde', (nt,))
    self.rest_vol = self._field('rest_vol', (nt,))
    self.Dm_inv = self._field('Dm_inv', (nt, 3, 3))
    self.v_p_old = self._field('v_p_old', (nv, 3))
    self.v_predict = self._field('v_predict', (nv, 3))
    self.dpos = self._field('dpos', (nv, 3))
    self._b_gpu = self._field('b', (nt,))
    self._dlam_gpu = self._field('dlam', (nt,))
    from .mgpcg_gpu import GPUMultigridSolver
    self._gpu_solver = GPUMultigridSolver._from_handle(self)
    self._nnz = int(self._gpu_solver._gpu_As[0].nnz)
    self._inited = True

  @property
  def _alpha_tilde_np(self):
    return self.alpha_tilde.detach().cpu().numpy()

  @property
  def _A_indptr(self):
    return self._gpu_solver._gpu_As[0].indptr.cpu().numpy()

  @property
  def _A_indices(self):
    return self._gpu_solver._gpu_As[0].indices.cpu().numpy()

  def stats(self) -> dict:
    s = N.Stats()
    N.check(self._lib.mgpbd_get_stats(self._h, C.byref(s)), 'mgpbd_get_stats')
    nl = s.n_levels
    return {
        'newton_iters': s.newton_iters, 'cg_iters_total': s.cg_iters_total,
        'cg_iters_last': s.cg_iters_last, 'n_levels': nl, 'residual0': s.residual0,
        'residual': s.residual, 'omega_last': s.omega_last, 'status': s.status,
        'rows': list(s.rows[:nl]), 'nnz': list(s.nnz[:nl]),
        'cg_path': ('kernels', 'persistent', 'staged', 'primal', 'primal-staged')[s.cg_path],
        'cg_grid': s.cg_grid, 'cg_iters_warm': s.cg_iters_warm, 'cg_launches': s.cg_launches,
        'ms_warm': s.ms_warm, 'ms_dual': s.ms_dual, 'warm_amp': s.warm_amp,
        'warm_declined': s.warm_declined, 'learned_fallbacks': s.learned_fallbacks,
        'learned_rejected': s.learned_rejected, 'learned_solves': s.learned_solves,
        'coarse_energy_learned': s.coarse_energy_learned,
        'coarse_energy_plain': s.coarse_energy_plain,
    }

  # ---- row-kernel autotuner (no reference counterpart) ---------------- #
  def autotune(self, reps=5, cache=None):
    """Pick the CSR row-kernel tile shape (G lanes x U float4, code
    G*100+U) of every multigrid level by timing all candidates on the
    level's matrix.  With `cache` (a JSON file path) levels are keyed by GPU
    name, rows and nonzeros: when every level is found the cached shapes are
    set without timing; otherwise all levels are tuned and the file updated.
    Returns {level: code}."""
    import json
    import os
    st = self.stats()
    nl = st['n_levels']
    gpu = torch.cuda.get_device_name(self.v_p.device)
    keys = [f"{gpu}|{st['rows'][l]}|{st['nnz'][l]}" for l in range(nl)]
    table = {}
    if cache is not None and os.path.exists(cache):
      with open(cache) as f:
        table = json.load(f)
    if cache is not None and all(k in table for k in keys):
      for l, k in enumerate(keys):
        N.check(self._lib.mgpbd_set_level_row_shape(self._h, l, int(table[k]['code'])),
                'mgpbd_set_level_row_shape')
      return {l: int(table[k]['code']) for l, k in enumerate(keys)}
    self._stream()
    codes = (C.c_int32 * nl)()
    us = (C.c_float * nl)()
    N.check(self._lib.mgpbd_autotune_rows(self._h, int(reps), codes, us), 'mgpbd_autotune_rows')
    self.last_tuning = {l: (int(codes[l]), float(us[l])) for l in range(nl)}
    if cache is not None:
      for l, k in enumerate(keys):
        table[k] = {'code': int(codes[l]), 'us_per_sweep': float(us[l])}
      tmp = cache + '.tmp'
      with open(tmp, 'w') as f:
        json.dump(table, f, indent=1, sort_keys=True)
      os.replace(tmp, cache)
    return {l: int(codes[l]) for l in range(nl)}

  def row_shape(self, level):
    """The row-kernel shape code of a level (0: from the mean row length)."""
    c = C.c_int32()
    N.check(self._lib.mgpbd_level_row_shape(self._h, int(level), C.byref(c)),
            'mgpbd_level_row_shape')
    return c.value

  def set_row_shape(self, level, code):
    N.check(self._lib.mgpbd_set_level_row_shape(self._h, int(level), int(code)),
            'mgpbd_set_level_row_shape')

  # ---- learned coarse correction (no reference counterpart) ----------- #
  def set_coarse_net(self, net):
    """Attach a trained `CoarseNet` (or None) for precond='learned'; the
    solver keeps a reference so the network outlives its use."""
    self._coarse_net = net
    N.check(self._lib.mgpbd_set_coarse_net(self._h, net._h if net is not None else None),
            'mgpbd_set_coarse_net')

  def record_coarse(self, capacity, every=1):
    """Start recording (restricted residual, plain coarse correction) pairs
    of level 1 from the plain V-cycles of the following solves; returns the
    two (capacity, n1) device buffers being filled."""
    n1 = int(self.stats()['rows'][1]) if self._inited else 0
    if n1 == 0:
      raise RuntimeError('record_coarse needs init() and a two-level hierarchy')
    rc = torch.zeros((capacity, n1), dtype=torch.float32, device=self.v_p.device)
    ec = torch.zeros_like(rc)
    self._rec = (rc, ec)
    N.check(self._lib.mgpbd_record_coarse(self._h, rc.data_ptr(), ec.data_ptr(), int(capacity),
                                          int(every)), 'mgpbd_record_coarse')
    return rc, ec

  def recorded_coarse(self):
    """The pairs stored so far: (rc[:k], ec[:k]); stops the recording."""
    k = C.c_int32()
    N.check(self._lib.mgpbd_record_count(self._h, C.byref(k)), 'mgpbd_record_count')
    N.check(self._lib.mgpbd_record_coarse(self._h, None, None, 0, 1), 'mgpbd_record_coarse')
    rc, ec = self._rec
    return rc[:k.value], ec[:k.value]

  def coarse_graph(self):
    """The level-1 aggregate graph (CSR + 1/diag, device tensors) that the
    learned coarse correction runs on."""
    from .learned import CoarseGraph
    return CoarseGraph.from_solver(self, 1)

  def newton_log(self):
    n = C.c_int32()
    N.check(self._lib.mgpbd_newton_log(self._h, 0, None, C.byref(n)), 'mgpbd_newton_log')
    rows = np.zeros((max(n.value, 1), 5), np.float64)
    N.check(self._lib.mgpbd_newton_log(self._h, n.value, rows.ctypes.data, C.byref(n)),
            'mgpbd_newton_log')
    return rows[:n.value]

  def _check(self, rc, where):
    if rc == -5 and not self.check_finite:
      return
    N.check(rc, where)

  # ------------------------------------------------------------------ #
  # cons/mgpbd_gpu.py:200-219
  def step(self, frame: int = 0):
    self.make_prediction()
    self.solve(frame)
    self.update_vel()

  def make_prediction(self):
    self._stream()
    N.check(self._lib.mgpbd_make_prediction(self._h), 'mgpbd_make_prediction')

  def update_vel(self):
    self._stream()
    N.check(self._lib.mgpbd_update_vel(self._h), 'mgpbd_update_vel')

  # cons/mgpbd_gpu.py:397-446
  def solve(self, frame: int = 0):
    self._stream()
    if self.benchmark is not None:
      self.benchmark.begin_frame(frame)
    rc = self._lib.mgpbd_solve(self._h, int(frame))
    if self.benchmark is not None:
      for ite, r, cg, om, t in self.newton_log():
        try:
          self.benchmark.record_iteration(int(ite), r, cg_iters=int(cg), omega=om, t=t)
        except TypeError:  # a recorder without the timestamp argument
          self.benchmark.record_iteration(int(ite), r, cg_iters=int(cg), omega=om)
      self.benchmark.end_frame()
    self._check(rc, 'mgpbd_solve')

  # ---- per-stage methods under the reference's names ------------------ #
  def _compute_C_and_gradC(self):
    self._stream()
    N.check(self._lib.mgpbd_compute_constraints(self._h), 'mgpbd_compute_constraints')

  def _residual_norm_gpu(self) -> float:
    self._stream()
    r = C.c_double()
    N.check(self._lib.mgpbd_compute_rhs(self._h, C.byref(r)), 'mgpbd_compute_rhs')
    return r.value

  def _compute_rhs_gpu(self):
    self._residual_norm_gpu()

  def _fill_A_and_update_gpu(self):
    self._stream()
    N.check(self._lib.mgpbd_fill_matrices(self._h), 'mgpbd_fill_matrices')

  def _zero_dpos(self):
    self.dpos.zero_()

  def _scatter_dlam_gpu(self):
    self._stream()
    N.check(self._lib.mgpbd_scatter(self._h, self._dlam_gpu.data_ptr()), 'mgpbd_scatter')

  def _line_search(self, beta=0.5, max_steps=10):
    if beta != 0.5 or max_steps != 10:
      raise NotImplementedError('the line search uses beta=0.5, max_steps=10 (reference defaults)')
    self._stream()
    w = C.c_double()
    N.check(self._lib.mgpbd_line_search(self._h, C.byref(w)), 'mgpbd_line_search')
    return w.value

  def _apply_dpos(self, omega: float):
    self._stream()
    N.check(self._lib.mgpbd_apply_dpos(self._h, float(omega)), 'mgpbd_apply_dpos')

  def synchronize(self):
    N.check(self._lib.mgpbd_synchronize(self._h), 'mgpbd_synchronize')

  def apply_A(self, x, matrix_free=True):
    """y = A x for the current system (matrix-free from the gradients, or
    with the assembled CSR values)."""
    self._stream()
    y = torch.empty_like(x)
    mode = int(matrix_free) if not isinstance(matrix_free, bool) else int(matrix_free)
    N.check(self._lib.mgpbd_apply_matrix(self._h, mode, x.data_ptr(), y.data_ptr()),
            'mgpbd_apply_matrix')
    return y

  def level_sweep(self, level, op, x, b=None, y=None, omega=2.0 / 3.0):
    """One pass of the internal CSR row kernel on a multigrid level."""
    self._stream()
    if y is None:
      y = torch.empty_like(x)
    N.check(self._lib.mgpbd_level_sweep(self._h, int(level), int(op), x.data_ptr(),
                                        b.data_ptr() if b is not None else None, y.data_ptr(),
                                        float(omega)), 'mgpbd_level_sweep')
    return y


def _now():
  return time.perf_counter()
