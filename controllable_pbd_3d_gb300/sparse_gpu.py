"""GPU CSR matrix and vector kernels with the API of the reference's
`cons/sparse_gpu.py` (free functions `gpu_dot` ... `gpu_negate_and_add`,
class `GPUSparseMatrix`), running the CUDA kernels of libmgpbd.so.

Vectors are float32 CUDA tensors.  Reductions accumulate in float64 in a
fixed order (the reference sums with float32 atomics in no fixed order).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as N


def _s():
  return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _f32(t):
  if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
    raise TypeError('expected a contiguous float32 CUDA tensor')
  return t


def gpu_dot(a, b, n) -> float:
  """cons/sparse_gpu.py:18-23"""
  out = C.c_double()
  N.check(N.lib().mgpbd_dot(int(n), _f32(a).data_ptr(), _f32(b).data_ptr(), C.byref(out), _s()),
          'mgpbd_dot')
  return out.value


def gpu_axpy(alpha, x, y, n):
  """cons/sparse_gpu.py:26-30: y += alpha x"""
  N.check(N.lib().mgpbd_axpy(int(n), float(alpha), _f32(x).data_ptr(), _f32(y).data_ptr(), _s()),
          'mgpbd_axpy')


def gpu_xpay(alpha, x, y, n):
  """cons/sparse_gpu.py:33-37: y = x + alpha y"""
  N.check(N.lib().mgpbd_xpay(int(n), float(alpha), _f32(x).data_ptr(), _f32(y).data_ptr(), _s()),
          'mgpbd_xpay')


def gpu_copy(src, dst, n):
  """cons/sparse_gpu.py:40-43 (a device-to-device copy)"""
  _f32(dst)[:n].copy_(_f32(src)[:n])


def gpu_fill_zero(x, n):
  """cons/sparse_gpu.py:46-49"""
  _f32(x)[:n].zero_()


def gpu_scale(x, alpha, n):
  """cons/sparse_gpu.py:52-55: x *= alpha"""
  N.check(N.lib().mgpbd_scale(int(n), float(alpha), _f32(x).data_ptr(), _s()), 'mgpbd_scale')


def gpu_norm_sq(x, n) -> float:
  """cons/sparse_gpu.py:58-63"""
  return gpu_dot(x, x, n)


def gpu_negate_and_add(b, r, n):
  """cons/sparse_gpu.py:66-70: r = b - r"""
  gpu_xpay(-1.0, b, r, n)


class GPUSparseMatrix:
  """CSR matrix in device memory (cons/sparse_gpu.py:78-144)."""

  def __init__(self, n_rows: int, nnz: int, _views=None):
    self.n_rows = int(n_rows)
    self.nnz = int(nnz)
    if _views is not None:
      self.indptr, self.indices, self.data, self.diag_inv = _views
      return
    self.data = torch.zeros(self.nnz, dtype=torch.float32, device='cuda')
    self.indices = torch.zeros(self.nnz, dtype=torch.int32, device='cuda')
    self.indptr = torch.zeros(self.n_rows + 1, dtype=torch.int32, device='cuda')
    self.diag_inv = torch.zeros(self.n_rows, dtype=torch.float32, device='cuda')

  def from_scipy(self, A: sp.csr_matrix):
    """Load pattern and values, keeping the given column order."""
    A = A.tocsr()
    assert A.shape[0] == self.n_rows
    assert A.nnz == self.nnz
    self.data.copy_(torch.from_numpy(np.asarray(A.data, np.float32)))
    self.indices.copy_(torch.from_numpy(np.asarray(A.indices, np.int32)))
    self.indptr.copy_(torch.from_numpy(np.asarray(A.indptr, np.int32)))
    self.cache_diag_inv()

  def update_data(self, data_np):
    self.data.copy_(torch.from_numpy(np.asarray(data_np, np.float32)))

  def cache_diag_inv(self):
    N.check(N.lib().mgpbd_csr_diag_inv(self.n_rows, self.indptr.data_ptr(), self.indices.data_ptr(),
                                       self.data.data_ptr(), self.diag_inv.data_ptr(), _s()),
            'mgpbd_csr_diag_inv')

  def spmv(self, x, y):
    N.check(N.lib().mgpbd_csr_spmv(self.n_rows, self.indptr.data_ptr(), self.indices.data_ptr(),
                                   self.data.data_ptr(), _f32(x).data_ptr(), _f32(y).data_ptr(),
                                   _s()), 'mgpbd_csr_spmv')

  def jacobi_smooth(self, b, x, x_new, omega):
    N.check(N.lib().mgpbd_csr_jacobi(self.n_rows, self.indptr.data_ptr(), self.indices.data_ptr(),
                                     self.data.data_ptr(), self.diag_inv.data_ptr(),
                                     _f32(b).data_ptr(), _f32(x).data_ptr(), _f32(x_new).data_ptr(),
                                     float(omega), _s()), 'mgpbd_csr_jacobi')

  def to_scipy(self):
    return sp.csr_matrix((self.data.cpu().numpy(), self.indices.cpu().numpy(),
                          self.indptr.cpu().numpy()), shape=(self.n_rows, self.n_rows))
