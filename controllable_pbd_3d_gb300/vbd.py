"""`VBDSolver`: Vertex Block Descent with the constructor, fields and
methods of the reference's `cons/vbd.py:6-361`, running on libmgpbd.so.

Methods (`method=`):
  'serial'  vertices one at a time in index order (one warp walks the
            vertices; its lanes split each vertex's incident tets);
  'color'   colour by colour (greedy vertex colouring), the vertices of a
            colour at once, 4 lanes per vertex; the whole solve
            (n_iterations x colours, plus the Chebyshev steps) is one
            cooperative kernel with grid barriers.

`v_p` (NV,3) float32 CUDA tensor is updated in place; `v_p_ref`, `v_invm`
and `t_i` are read by the library (kept referenced here).  `t_m` is stored
like the reference stores it; the solver does not use it.  After
construction `v_v`, `v_p_old`, `x_tilde`, `Dm_inv` and `rest_vol` are
torch views of the library's memory.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .graph_coloring import color_vertices
from .mgpbd_gpu import _cuda, _Scalar, device_view


class VBDSolver:
  """cons/vbd.py:6-361."""

  def __init__(self, v_p, v_p_ref, v_invm, t_i, t_m, gravity, dt: float, damp: float = 1.0,
               youngs_modulus: float = 1e4, poissons_ratio: float = 0.3, damping: float = 0.0,
               n_iterations: int = 10, rho: float = 0.0, method: str = 'serial',
               benchmark=None) -> None:
    if method not in N.VBD_METHOD:
      raise ValueError(f"unknown VBD method '{method}' (one of {list(N.VBD_METHOD)})")
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
    g = gravity.to_numpy() if hasattr(gravity, 'to_numpy') else gravity
    self.gravity = [float(v) for v in g]
    self.dt = float(dt)
    self.n_iterations = int(n_iterations)
    self.rho = float(rho)
    self.damping_coeff = float(damping)
    self.method = method
    self.benchmark = benchmark
    self.damp = _Scalar(damp)
    p = N.VbdParams(dt=self.dt, damp=float(damp), youngs_modulus=float(youngs_modulus),
                    poissons_ratio=float(poissons_ratio), damping=self.damping_coeff,
                    rho=self.rho, gravity=(C.c_float * 3)(*self.gravity),
                    n_iterations=self.n_iterations, method=N.VBD_METHOD[method])
    h = C.c_void_p()
    N.check(self._lib.mgpbd_vbd_create(C.byref(p), C.byref(h)), 'mgpbd_vbd_create')
    self._h = h
    self._stream()
    N.check(self._lib.mgpbd_vbd_set_mesh(self._h, self.v_p.data_ptr(), self.v_p_ref.data_ptr(),
                                         self.v_invm.data_ptr(), self.t_i.data_ptr(),
                                         self.n_verts, self.n_tets), 'mgpbd_vbd_set_mesh')
    mu, lam = C.c_float(), C.c_float()
    N.check(self._lib.mgpbd_vbd_lame(self._h, C.byref(mu), C.byref(lam)), 'mgpbd_vbd_lame')
    self.mu, self.lam = float(mu.value), float(lam.value)
    om = np.empty(max(self.n_iterations, 1), np.float32)
    N.check(self._lib.mgpbd_vbd_omegas(self._h, om.ctypes.data), 'mgpbd_vbd_omegas')
    self._omegas = [float(v) for v in om[:self.n_iterations]]
    self.v_v = self._field('v_v', (self.n_verts, 3))
    self.v_p_old = self._field('v_p_old', (self.n_verts, 3))
    self.x_tilde = self._field('x_tilde', (self.n_verts, 3))
    self.Dm_inv = self._field('Dm_inv', (self.n_tets, 3, 3))
    self.rest_vol = self._field('rest_vol', (self.n_tets,))
    if method == 'color':
      self._compute_vertex_coloring()

  def _field(self, name, shape):
    ptr, cnt = C.c_void_p(), C.c_int64()
    N.check(self._lib.mgpbd_vbd_field(self._h, N.VBD_FIELD[name], C.byref(ptr), C.byref(cnt)),
            'mgpbd_vbd_field')
    return device_view(ptr.value, shape)

  def _stream(self):
    N.check(self._lib.mgpbd_vbd_set_stream(self._h, torch.cuda.current_stream().cuda_stream),
            'mgpbd_vbd_set_stream')

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      self._lib.mgpbd_vbd_destroy(h)
      self._h = None

  # cons/vbd.py:98-104 (the library colours the vertices the same way)
  def _compute_vertex_coloring(self):
    res = color_vertices(self.t_i.cpu().numpy(), self.n_tets, 4, self.n_verts)
    self.color_offsets = res.color_offsets
    self.color_vertex_order = torch.as_tensor(res.ordered_indices, device='cuda')
    self.num_colors = res.num_colors

  def init(self):
    self._stream()
    N.check(self._lib.mgpbd_vbd_init(self._h), 'mgpbd_vbd_init')

  def make_prediction(self):
    self._stream()
    N.check(self._lib.mgpbd_vbd_make_prediction(self._h), 'mgpbd_vbd_make_prediction')

  # cons/vbd.py:134-160: the iterations run in one launch; the benchmark
  # gets one record per iteration (omega as the reference records it) with
  # the time at the end of the solve
  def solve(self, frame: int = 0):
    if self.benchmark is not None:
      self.benchmark.begin_frame(frame)
    self._stream()
    N.check(self._lib.mgpbd_vbd_solve(self._h), 'mgpbd_vbd_solve')
    if self.benchmark is not None:
      for n, om in enumerate(self._omegas):
        self.benchmark.record_iteration(n, 0.0, omega=om)
      self.benchmark.end_frame()

  def synchronize(self):
    """Wait for the queued solve and raise if the colour kernel's grid
    barrier gave up."""
    N.check(self._lib.mgpbd_vbd_synchronize(self._h), 'mgpbd_vbd_synchronize')

  def update_vel(self):
    self._stream()
    N.check(self._lib.mgpbd_vbd_update_vel(self._h), 'mgpbd_vbd_update_vel')

  def step(self, frame: int = 0):
    self.make_prediction()
    self.solve(frame)
    self.update_vel()
