"""`Deform3D`: local XPBD with one coupled hydrostatic (det F - 1) and
deviatoric (|F|^2 - 3) constraint per tet, with the constructor and
`pbd_framework` protocol of the reference's `cons/deform3d.py:7-288`,
running on libmgpbd.so.

Methods (`method=`):
  'default'         every tet at once, position updates by atomic adds that
                    race with other tets' reads (the reference's parallel
                    loop; not deterministic);
  'gauss_seidel'    one tet at a time in index order (one GPU thread);
  'graph_coloring'  colour by colour (greedy tet colouring), the tets of a
                    colour at once; one cooperative kernel per pass with a
                    grid barrier between colours; deterministic.

Inputs are CUDA tensors (or arrays, copied to the GPU): `v_p` (NV,3)
float32 is updated in place; `v_p_ref`, `v_invm`, `t_i` (4*NT int32) and
`t_m` (NT) are read by the library during every pass, so they must stay
alive (the object keeps references).
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _native as N
from .graph_coloring import color_elements
from .mgpbd_gpu import _cuda, device_view


class Deform3D:
  """cons/deform3d.py:7-288."""

  def __init__(self, v_p, v_p_ref, v_invm, t_i, t_m, dt: float, hydro_alpha=0.0,
               devia_alpha=0.0, method='default', benchmark=None) -> None:
    if method not in N.XPBD_METHOD:
      raise ValueError(f"unknown Deform3D method '{method}' (one of {list(N.XPBD_METHOD)})")
    self._lib = N.lib()
    self.v_p = _cuda(v_p, torch.float32, (-1, 3))
    if isinstance(v_p, torch.Tensor) and self.v_p.data_ptr() != v_p.data_ptr():
      raise ValueError('v_p must be a contiguous float32 CUDA tensor (it is updated in place)')
    self.v_p_ref = _cuda(v_p_ref, torch.float32, (-1, 3))
    self.v_invm = _cuda(v_invm, torch.float32, (-1,))
    self.t_i = _cuda(t_i, torch.int32, (-1,))
    self.t_m = _cuda(t_m, torch.float32, (-1,))
    self.n = self.t_i.shape[0] // 4
    if self.t_m.shape[0] != self.n:
      raise ValueError('t_m must hold one mass per tet')
    self.hydro_alpha = float(hydro_alpha)
    self.devia_alpha = float(devia_alpha)
    self.dt = float(dt)
    self.method = method
    self.benchmark = benchmark
    self._update_count = 0
    p = N.XpbdParams(dt=self.dt, hydro_alpha=self.hydro_alpha, devia_alpha=self.devia_alpha,
                     method=N.XPBD_METHOD[method])
    h = C.c_void_p()
    N.check(self._lib.mgpbd_xpbd_create(C.byref(p), C.byref(h)), 'mgpbd_xpbd_create')
    self._h = h
    self._stream()
    N.check(self._lib.mgpbd_xpbd_set_mesh(self._h, self.v_p.data_ptr(), self.v_p_ref.data_ptr(),
                                          self.v_invm.data_ptr(), self.t_i.data_ptr(),
                                          self.t_m.data_ptr(), self.v_p.shape[0], self.n),
            'mgpbd_xpbd_set_mesh')
    hp, dp = C.c_void_p(), C.c_void_p()
    N.check(self._lib.mgpbd_xpbd_lambdas(self._h, C.byref(hp), C.byref(dp)), 'mgpbd_xpbd_lambdas')
    self.hydro_lambda = device_view(hp.value, (self.n,))
    self.devia_lambda = device_view(dp.value, (self.n,))
    if method == 'graph_coloring':
      self.compute_graph_coloring()

  def _stream(self):
    N.check(self._lib.mgpbd_xpbd_set_stream(self._h, torch.cuda.current_stream().cuda_stream),
            'mgpbd_xpbd_set_stream')

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      self._lib.mgpbd_xpbd_destroy(h)
      self._h = None

  # cons/deform3d.py:202-208 (the library colours the tets the same way)
  def compute_graph_coloring(self):
    res = color_elements(self.t_i.cpu().numpy(), self.n, 4, self.v_p.shape[0])
    self.colored_tet_order = torch.as_tensor(res.ordered_indices, device='cuda')
    self.color_offsets = res.color_offsets
    self.num_colors = res.num_colors

  # cons/deform3d.py:37-42
  def init_rest_status(self):
    pass

  def preupdate_cons(self):
    self._stream()
    N.check(self._lib.mgpbd_xpbd_preupdate(self._h), 'mgpbd_xpbd_preupdate')

  def synchronize(self):
    """Wait for the queued passes and raise if a colour kernel's grid
    barrier gave up (passes are asynchronous on the current stream)."""
    N.check(self._lib.mgpbd_xpbd_synchronize(self._h), 'mgpbd_xpbd_synchronize')

  # cons/deform3d.py:44-52
  def update_cons(self, n_passes: int = 1):
    self._stream()
    N.check(self._lib.mgpbd_xpbd_update(self._h, int(n_passes)), 'mgpbd_xpbd_update')
    if self.benchmark is not None:
      for _ in range(int(n_passes)):
        self.benchmark.record_iteration(self._update_count, 0.0)
        self._update_count += 1
