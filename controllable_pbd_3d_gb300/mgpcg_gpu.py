"""`GPUMultigridSolver` with the methods of the reference's
`cons/mgpcg_gpu.py:17-329` (`setup`, `solve`, `vcycle`,
`update_fine_matrix_data`, `update_all_coarse_matrices`, `_gpu_As`,
`_level_sizes`).

Two ways to get one: standalone, `GPUMultigridSolver(n_smooth,
omega_jacobi, maxiter_cg, tol_cg).setup(A, Ps)` with the caller's scipy
level-0 matrix and prolongations (a libmgpbd.so handle in matrix mode,
`mgpbd_set_matrix`); or bound to the hierarchy an `MGPBDSolverGPU` built
from its mesh (`solver._gpu_solver`)."""

from __future__ import annotations

import ctypes as C

import torch

from . import _native as N
from .sparse_gpu import GPUSparseMatrix


class GPUMultigridSolver:
  """V-cycle-preconditioned CG on the hierarchy of one MGPBD solver."""

  def __init__(self, n_smooth: int = 2, omega_jacobi: float = 2.0 / 3.0, maxiter_cg: int = 100,
               tol_cg: float = 1e-5):
    self.n_smooth = n_smooth
    self.omega_jacobi = omega_jacobi
    self.maxiter_cg = maxiter_cg
    self.tol_cg = tol_cg
    self.n_levels = 0
    self._solver = None
    self._h = None
    self._lib = N.lib()

  def __del__(self):
    if self._solver is None and getattr(self, '_h', None) is not None and self._h.value:
      try:
        self._lib.mgpbd_destroy(self._h)
      except Exception:
        pass
      self._h = None

  @staticmethod
  def _aggregates(P, n_fine):
    """Aggregate ids of an aggregation prolongation (one 1 per row)."""
    import numpy as np
    P = P.tocsr()
    if P.shape[0] != n_fine:
      raise ValueError(f'P has {P.shape[0]} rows, the level above has {n_fine}')
    P.sum_duplicates()
    if not (np.all(np.diff(P.indptr) == 1) and np.all(P.data == 1)):
      raise ValueError('each P must have exactly one entry, 1, per row (aggregation '
                       'prolongation, as cons/tet_aggregation.py builds)')
    return np.asarray(P.indices, np.int32), int(P.shape[1])

  def setup(self, A_level0_scipy, Ps_scipy: list):
    """cons/mgpcg_gpu.py:30-173: the hierarchy of A (scipy sparse, float32
    values, every row with its diagonal) under the prolongations Ps
    (aggregation operators: one 1 per row), Galerkin coarse levels and
    their contribution maps built by libmgpbd.so."""
    import numpy as np
    A = A_level0_scipy.tocsr()
    n = A.shape[0]
    if A.shape[1] != n:
      raise ValueError('A must be square')
    p = N.default_params()
    p.dt = 1.0  # no time stepping on a caller's matrix; the field must be valid
    p.n_smooth = int(self.n_smooth)
    p.omega_jacobi = float(self.omega_jacobi)
    p.maxiter_cg = int(self.maxiter_cg)
    p.tol_cg = float(self.tol_cg)
    if self._h is not None and self._h.value:
      self._lib.mgpbd_destroy(self._h)
    h = C.c_void_p()
    N.check(self._lib.mgpbd_create(C.byref(p), C.byref(h)), 'mgpbd_create')
    self._h = h
    self._params = p
    self._stream()
    ip = np.ascontiguousarray(A.indptr, np.int32)
    ix = np.ascontiguousarray(A.indices, np.int32)
    d = np.ascontiguousarray(A.data, np.float32)
    N.check(self._lib.mgpbd_set_matrix(h, n, len(ix), ip.ctypes.data, ix.ctypes.data,
                                       d.ctypes.data), 'mgpbd_set_matrix')
    if Ps_scipy:
      sizes, aggs = [n], []
      for P in Ps_scipy:
        a, nc = self._aggregates(P, sizes[-1])
        aggs.append(a)
        sizes.append(nc)
      flat = np.ascontiguousarray(np.concatenate(aggs))
      sz = np.asarray(sizes, np.int32)
      N.check(self._lib.mgpbd_set_hierarchy(h, flat.ctypes.data, len(sizes), sz.ctypes.data),
              'mgpbd_set_hierarchy')
    N.check(self._lib.mgpbd_init(h), 'mgpbd_init')
    self._bind()
    return self

  def _stream(self):
    if self._solver is not None:
      self._solver._stream()
    else:
      N.check(self._lib.mgpbd_set_stream(
          self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)), 'mgpbd_set_stream')

  @classmethod
  def _from_handle(cls, solver):
    self = cls.__new__(cls)
    self._solver = solver
    self._h = solver._h
    self._lib = N.lib()
    p = solver.params
    self.n_smooth = p.n_smooth
    self.omega_jacobi = p.omega_jacobi
    self.maxiter_cg = p.maxiter_cg
    self.tol_cg = p.tol_cg
    self._bind()
    return self

  def _bind(self):
    """Views of the library's level matrices and aggregate maps."""
    nl = C.c_int32()
    N.check(self._lib.mgpbd_level_count(self._h, C.byref(nl)), 'mgpbd_level_count')
    self.n_levels = nl.value
    from .mgpbd_gpu import device_view
    self._gpu_As = []
    self._level_sizes = []
    self._agg = []
    for l in range(self.n_levels):
      n = C.c_int32()
      nnz = C.c_int64()
      ip, ix, d, di = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
      N.check(self._lib.mgpbd_level_csr(self._h, l, C.byref(n), C.byref(nnz), C.byref(ip),
                                        C.byref(ix), C.byref(d), C.byref(di)), 'mgpbd_level_csr')
      views = (device_view(ip.value, (n.value + 1,), torch.int32),
               device_view(ix.value, (nnz.value,), torch.int32),
               device_view(d.value, (nnz.value,)),
               device_view(di.value, (n.value,)))
      self._gpu_As.append(GPUSparseMatrix(n.value, nnz.value, _views=views))
      self._level_sizes.append(n.value)
      if l + 1 < self.n_levels:
        ag = C.c_void_p()
        N.check(self._lib.mgpbd_level_agg(self._h, l, C.byref(ag)), 'mgpbd_level_agg')
        self._agg.append(device_view(ag.value, (n.value,), torch.int32))

  def solve(self, b_field, x_field) -> int:
    """CG with the V-cycle preconditioner (cons/mgpcg_gpu.py:261-329);
    x_field is overwritten, the CG iteration count is returned."""
    self._stream()
    it = C.c_int32()
    N.check(self._lib.mgpbd_pcg(self._h, b_field.data_ptr(), x_field.data_ptr(), C.byref(it)),
            'mgpbd_pcg')
    return it.value

  def vcycle_apply(self, r):
    """z = V-cycle(r) from a zero initial guess (cons/mgpcg_gpu.py:214-259)."""
    self._stream()
    z = torch.empty_like(r)
    N.check(self._lib.mgpbd_vcycle(self._h, r.data_ptr(), z.data_ptr()), 'mgpbd_vcycle')
    return z

  def update_fine_matrix_data(self, data):
    """cons/mgpcg_gpu.py:175-181: copy level-0 values, refresh 1/diag (and,
    for a standalone solver, the coarse levels as well)."""
    A = self._gpu_As[0]
    vals = torch.as_tensor(data, dtype=torch.float32).reshape(-1).to(A.data.device)
    if self._solver is None:
      self._stream()
      vals = vals.contiguous()
      N.check(self._lib.mgpbd_update_matrix(self._h, vals.data_ptr()), 'mgpbd_update_matrix')
      return
    A.data.copy_(vals)
    A.cache_diag_inv()

  def update_all_coarse_matrices(self):
    """cons/mgpcg_gpu.py:200-212: coarse values by the contribution map."""
    self._stream()
    N.check(self._lib.mgpbd_refill_coarse(self._h), 'mgpbd_refill_coarse')
