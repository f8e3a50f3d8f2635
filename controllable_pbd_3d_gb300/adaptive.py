"""Spatial adaptivity around the MGPBD step: AdaptiveZone
(cons/adaptive_zone.py:14-91) and MGPBDAdaptiveSolver
(cons/mgpbd_adaptive.py:14-93), with the same methods and semantics, on the
library's zone kernels.

A zone holds one int32 flag per tet (1 active, 0 passive) as a CUDA tensor
`tet_active`.  Before each solve the adaptive solver raises alpha~ of the
passive tets to 1e20 (their constraints then exert no force) and restores
it afterwards, exactly like the reference wrapper.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .mgpbd_gpu import MGPBDSolverGPU


class AdaptiveZone:
  """Per-tet active/passive flags (cons/adaptive_zone.py:14-91).  The zone
  runs its kernels through a solver handle on the same mesh: pass `solver`
  here or let MGPBDAdaptiveSolver attach its own."""

  def __init__(self, n_tets: int, t_i=None, v_p=None, solver: MGPBDSolverGPU | None = None):
    self.n_tets = int(n_tets)
    self.t_i = t_i
    self.v_p = v_p
    self.solver = solver
    self.n_verts = int(v_p.shape[0]) if v_p is not None else None
    self.tet_active = torch.ones(self.n_tets, dtype=torch.int32, device='cuda')

  def _h(self):
    if self.solver is None:
      raise RuntimeError('AdaptiveZone needs a solver on the same mesh (solver=... or '
                         'MGPBDAdaptiveSolver)')
    if self.solver.n_tets != self.n_tets:
      raise ValueError('zone and solver have different tet counts')
    self.solver._stream()
    return self.solver._h

  # cons/adaptive_zone.py:40-55
  def update_by_proximity(self, tool_x: float, tool_y: float, tool_z: float, radius: float):
    N.check(N.lib().mgpbd_zone_proximity(self._h(), self.tet_active.data_ptr(), float(tool_x),
                                         float(tool_y), float(tool_z), float(radius)),
            'mgpbd_zone_proximity')

  # cons/adaptive_zone.py:57-72
  def update_by_strain(self, v_p_old, threshold: float, dt: float):
    h = self._h()
    ptr = None
    if v_p_old is not None:
      if not (isinstance(v_p_old, torch.Tensor) and v_p_old.is_cuda and
              v_p_old.dtype == torch.float32 and v_p_old.is_contiguous()):
        v_p_old = torch.as_tensor(np.asarray(v_p_old, np.float32), device='cuda').contiguous()
      self._x_old = v_p_old
      ptr = v_p_old.data_ptr()
    N.check(N.lib().mgpbd_zone_strain(h, self.tet_active.data_ptr(), ptr, float(threshold),
                                      float(dt)), 'mgpbd_zone_strain')

  # cons/adaptive_zone.py:74-85
  def expand_zone(self, n_rings: int):
    N.check(N.lib().mgpbd_zone_expand(self._h(), self.tet_active.data_ptr(), int(n_rings)),
            'mgpbd_zone_expand')

  def get_active_mask(self) -> np.ndarray:
    return self.tet_active.cpu().numpy().astype(bool)

  def get_active_fraction(self) -> float:
    return float(self.tet_active.sum().item()) / self.n_tets


class MGPBDAdaptiveSolver:
  """Wrapper that adds spatial adaptivity to an MGPBDSolverGPU
  (cons/mgpbd_adaptive.py:14-93)."""

  def __init__(self, solver: MGPBDSolverGPU, zone: AdaptiveZone, passive_iters: int = 2):
    self.solver = solver
    self.zone = zone
    if zone.solver is None:
      zone.solver = solver
    self.passive_iters = passive_iters
    self.n_tets = solver.n_tets
    self.n_verts = solver.n_verts
    self.v_p = solver.v_p
    self.v_v = solver.v_v
    self.v_p_old = solver.v_p_old
    self.damp = solver.damp
    self._original_alpha = torch.empty(self.n_tets, dtype=torch.float32, device='cuda')

  # cons/mgpbd_adaptive.py:36-62
  def step(self, frame: int = 0, tool_pos=None, tool_radius: float = 0.5):
    self.solver.make_prediction()
    if tool_pos is not None:
      self.zone.update_by_proximity(float(tool_pos[0]), float(tool_pos[1]), float(tool_pos[2]),
                                    float(tool_radius))
      self.zone.expand_zone(1)
    self._apply_active_mask()
    self.solver.solve(frame)
    self._restore_mask()
    self.solver.update_vel()

  def _apply_active_mask(self):
    self.solver._stream()
    N.check(N.lib().mgpbd_mask_alpha(self.solver._h, self.zone.tet_active.data_ptr(),
                                     self._original_alpha.data_ptr()), 'mgpbd_mask_alpha')

  def _restore_mask(self):
    self.solver._stream()
    N.check(N.lib().mgpbd_restore_alpha(self.solver._h, self._original_alpha.data_ptr()),
            'mgpbd_restore_alpha')


def host_face_adjacency(t_i, nt: int):
  """Face adjacency of cons/tet_aggregation.py:11-37 as CSR (host)."""
  t = np.ascontiguousarray(t_i, np.int32)
  nnz = C.c_int64()
  L = N.lib()
  N.check(L.mgpbd_host_face_adjacency(t.ctypes.data, int(nt), C.byref(nnz), None, None),
          'mgpbd_host_face_adjacency')
  ip = np.empty(nt + 1, np.int32)
  ix = np.empty(max(nnz.value, 1), np.int32)
  N.check(L.mgpbd_host_face_adjacency(t.ctypes.data, int(nt), C.byref(nnz), ip.ctypes.data,
                                      ix.ctypes.data), 'mgpbd_host_face_adjacency')
  return ip, ix[:nnz.value]
