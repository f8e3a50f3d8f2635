"""The MGPBD global step behind the constraint-solver interface of the
reference's `pbd_framework` (cons/framework.py:6-89).

`pbd_framework` owns the positions' prediction and the velocities and calls,
per substep, `preupdate_cons()` once and `update_cons()` `subsub` times on
every registered constraint object (cons/framework.py:73-89).  `MGPBDConstraint`
is such an object for the MGPBD step: `update_cons()` is one Newton
iteration of `MGPBDSolverGPU.solve` (cons/mgpbd_gpu.py:405-440) on the
framework's positions, in the library, and becomes a no-op once the Newton
stopping test (`atol`, `rtol` relative to the substep's first residual,
cons/mgpbd_gpu.py:412-416) holds.  `PbdFramework` mirrors the framework's
own loop (prediction, constraint passes, velocity update) over torch tensors
so the adapter can be driven without Taichi.
"""

from __future__ import annotations

import math

import torch

from .mgpbd_gpu import MGPBDSolverGPU


class MGPBDConstraint:
  """`pbd_framework` constraint protocol over an `MGPBDSolverGPU` whose
  positions tensor is the framework's `v_p`."""

  def __init__(self, solver: MGPBDSolverGPU):
    self.solver = solver
    self._r0 = None
    self._done = False
    self.ite = 0
    self.log = []

  # cons/framework.py:60-66
  def init_rest_status(self):
    if not self.solver._inited:
      self.solver.init()

  # cons/framework.py:68-76: a new substep starts from lambda = 0
  def preupdate_cons(self):
    self.solver.lambdaf.zero_()
    self._r0 = None
    self._done = False
    self.ite = 0
    self.log = []

  # cons/framework.py:78-82: one Newton iteration of cons/mgpbd_gpu.py:405-440
  def update_cons(self):
    if self._done:
      return
    s = self.solver
    p = s.params
    if self.ite >= p.maxiter:
      self._done = True
      return
    s._compute_C_and_gradC()
    r = s._residual_norm_gpu()
    if self._r0 is None:
      self._r0 = r
    if not math.isfinite(r):
      raise FloatingPointError(f'MGPBD residual is {r} at Newton iteration {self.ite}')
    if r < p.atol or (self._r0 > 1e-12 and r < p.rtol * self._r0):
      self._done = True
      self.log.append((self.ite, r, 0, 1.0))
      return
    s._fill_A_and_update_gpu()
    it = s._gpu_solver.solve(s._b_gpu, s._dlam_gpu)
    s._scatter_dlam_gpu()
    omega = s._line_search() if p.use_line_search else 1.0
    s._apply_dpos(omega)
    self.log.append((self.ite, r, it, omega))
    self.ite += 1


class PbdFramework:
  """The loop of cons/framework.py:6-89 over torch tensors: positions `v_p`
  (NV, 3) on the GPU (updated in place), velocities owned here."""

  def __init__(self, v_p: torch.Tensor, g, dt: float, damp: float = 1.0):
    self.v_p = v_p
    self.v_v = torch.zeros_like(v_p)
    self.v_p_cache = torch.zeros_like(v_p)
    self.g = torch.tensor(g, dtype=v_p.dtype, device=v_p.device)
    self.dt = float(dt)
    self.damp = float(damp)
    self.cons_list = [[]]

  def add_cons(self, new_cons, index=0):
    if index == len(self.cons_list):
      self.cons_list.append([])
    self.cons_list[index].append(new_cons)

  # cons/framework.py:28-35: every vertex is predicted (pinned ones too)
  def make_prediction(self):
    self.v_p_cache.copy_(self.v_p)
    self.v_p.add_(self.v_v * self.dt + self.g * (self.dt * self.dt))

  # cons/framework.py:37-42
  def update_vel(self):
    self.v_v.copy_(self.damp * (self.v_p - self.v_p_cache) / self.dt)

  def init_rest_status(self, index=0):
    for c in self.cons_list[index]:
      c.init_rest_status()

  def preupdate_cons(self, index=0):
    for c in self.cons_list[index]:
      c.preupdate_cons()

  def update_cons(self, index=0):
    for c in self.cons_list[index]:
      c.update_cons()

  # cons/framework.py:84-89
  def step(self, subsub=1, index=0):
    self.make_prediction()
    self.preupdate_cons(index)
    for _ in range(subsub):
      self.update_cons(index)
    self.update_vel()
