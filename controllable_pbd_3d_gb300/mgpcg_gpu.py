"""`GPUMultigridSolver` view with the methods of the reference's
`cons/mgpcg_gpu.py:17-329` (`solve`, `vcycle`, `update_fine_matrix_data`,
`update_all_coarse_matrices`, `_gpu_As`, `_level_sizes`), bound to the
hierarchy an `MGPBDSolverGPU` built in libmgpbd.so."""

from __future__ import annotations

import ctypes as C

import torch

from . import _native as N
from .sparse_gpu import GPUSparseMatrix


class GPUMultigridSolver:
  """V-cycle-preconditioned CG on the hierarchy of one MGPBD solver."""

  def __init__(self, n_smooth: int = 2, omega_jacobi: float = 2.0 / 3.0, maxiter_cg: int = 100,
               tol_cg: float = 1e-5):
    raise NotImplementedError(
        'GPUMultigridSolver is created by MGPBDSolverGPU.init() (solver._gpu_solver); the '
        'hierarchy is built from the tet mesh by libmgpbd.so')

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
    return self

  def solve(self, b_field, x_field) -> int:
    """CG with the V-cycle preconditioner (cons/mgpcg_gpu.py:261-329)."""
    self._solver._stream()
    it = C.c_int32()
    N.check(self._lib.mgpbd_pcg(self._h, b_field.data_ptr(), x_field.data_ptr(), C.byref(it)),
            'mgpbd_pcg')
    return it.value

  def vcycle_apply(self, r):
    """z = V-cycle(r) from a zero initial guess (cons/mgpcg_gpu.py:214-259)."""
    self._solver._stream()
    z = torch.empty_like(r)
    N.check(self._lib.mgpbd_vcycle(self._h, r.data_ptr(), z.data_ptr()), 'mgpbd_vcycle')
    return z

  def update_fine_matrix_data(self, data):
    """cons/mgpcg_gpu.py:175-181: copy level-0 values, refresh 1/diag."""
    A = self._gpu_As[0]
    A.data.copy_(torch.as_tensor(data, dtype=torch.float32).reshape(-1).to(A.data.device))
    A.cache_diag_inv()

  def update_all_coarse_matrices(self):
    """cons/mgpcg_gpu.py:200-212: coarse values by the contribution map."""
    self._solver._stream()
    N.check(self._lib.mgpbd_refill_coarse(self._h), 'mgpbd_refill_coarse')
