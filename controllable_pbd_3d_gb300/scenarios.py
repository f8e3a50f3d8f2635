"""Seeded scenarios of the benchmark configuration (input generation and
host-side drivers only; the step itself runs in libmgpbd.so).

`drag_slab` is the stiff-drag case: an nx x ny x nz hex slab (5 tets per
hex), one long edge pinned, the opposite corner vertex dragged along +z.
Dragging follows the reference's mechanism (`experiments/exp_tool_tissue.py`,
`experiments/exp_adaptive.py`): the dragged vertex is a pinned vertex
(inverse mass 0, kinematic) whose position the host overwrites before each
frame, and the solve pulls the body after it.
"""

from __future__ import annotations

import numpy as np
import torch

from . import meshgen


def cube_body(n, seed=0):
  """The benchmark's cube: n x n x n hexes of side 1/n (5 tets per hex), start
  positions jittered U(+-0.01 h) from `seed`, unit vertex mass, the top face
  (max y) pinned, compliance log-uniform in [1e-9, 1e-4] drawn from a fresh
  `default_rng(seed)`.  Returns (x_ref, x0, t_i, invm, compliance)."""
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=0.01, seed=seed)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  compliance = float(10.0 ** np.random.default_rng(seed).uniform(-9.0, -4.0))
  return xr, x0, t, invm, compliance


def grid_edge_vertices(nx, ny, nz, j=0, k=0):
  """Vertex ids of the grid line along x at (y index j, z index k)."""
  i = np.arange(nx + 1)
  return (i + (nx + 1) * (j + (ny + 1) * k)).astype(np.int64)


def drag_slab(nx=100, ny=25, nz=100, h=None, jitter=0.0, seed=0):
  """The slab, its pinned long edge (y = 0, z = 0, along x) and the dragged
  corner (x, y, z max).  Returns dict(x_ref, x0, t_i, invm, pinned, drag)."""
  xr, t = meshgen.hex_grid_tets(nx, ny, nz, h=h)
  x0, _ = meshgen.hex_grid_tets(nx, ny, nz, h=h, jitter=jitter, seed=seed) if jitter else (xr, t)
  pinned = grid_edge_vertices(nx, ny, nz, 0, 0)
  drag = int(nx + (nx + 1) * (ny + (ny + 1) * nz))
  invm = np.ones(len(xr), np.float32)
  invm[pinned] = 0.0
  invm[drag] = 0.0
  return dict(x_ref=xr.astype(np.float32), x0=x0.astype(np.float32), t_i=t.astype(np.int32),
              invm=invm, pinned=pinned, drag=drag)


class DragDriver:
  """Moves the dragged vertex of `solver` (an MGPBDSolverGPU with
  kinematic_pins=True) by `distance` along `direction` over `frames`
  frames, linearly, before each frame's substeps."""

  def __init__(self, solver, vertex, distance=0.5, frames=60, direction=(0.0, 0.0, 1.0)):
    self.solver = solver
    self.vertex = int(vertex)
    self.start = solver.v_p[self.vertex].detach().clone()
    d = torch.tensor(direction, dtype=torch.float32, device=solver.v_p.device)
    self.step_vec = d / torch.linalg.norm(d) * (float(distance) / int(frames))
    self.frames = int(frames)

  def target(self, frame):
    return self.start + self.step_vec * min(int(frame) + 1, self.frames)

  def frame(self, frame, substeps=5):
    with torch.no_grad():
      self.solver.v_p[self.vertex] = self.target(frame)
    for _ in range(substeps):
      self.solver.step(frame)


def grid_surface_vertices(nx, ny, nz):
  """Ids of the grid's boundary vertices (by index, robust to jitter and to
  the ball projection)."""
  ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                           indexing='ij')
  on = (ii == 0) | (ii == nx) | (jj == 0) | (jj == ny) | (kk == 0) | (kk == nz)
  vid = ii + (nx + 1) * (jj + (ny + 1) * kk)
  return np.sort(vid[on]).astype(np.int64)


def training_body(rng, sides=(20, 40), compliance=(1e-9, 1e-4), pinned=(0.01, 0.04),
                  jitter=0.01):
  """One body of the learned preconditioner's training set: a hex-grid cube
  (5 tets per hex) with side count uniform in `sides`, with probability 1/2
  radially projected onto its ball, compliance log-uniform in `compliance`,
  and a fraction uniform in `pinned` of its surface vertices pinned at
  random.  Returns dict(x_ref, x0, t_i, invm, compliance, side, ball,
  pinned)."""
  n = int(rng.integers(sides[0], sides[1] + 1))
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=jitter, seed=int(rng.integers(1 << 31)))
  ball = bool(rng.random() < 0.5)
  if ball:
    # project the rest shape and the jittered start with the same centre
    c = 0.5 * (xr.min(axis=0) + xr.max(axis=0))
    xr = meshgen.ball_project(xr, c)
    x0 = meshgen.ball_project(x0, c)
  surf = grid_surface_vertices(n, n, n)
  k = max(1, int(round(rng.uniform(*pinned) * len(surf))))
  pin = np.sort(rng.choice(surf, size=k, replace=False))
  invm = np.ones(len(xr), np.float32)
  invm[pin] = 0.0
  comp = float(10.0 ** rng.uniform(np.log10(compliance[0]), np.log10(compliance[1])))
  return dict(x_ref=xr.astype(np.float32), x0=x0.astype(np.float32), t_i=t.astype(np.int32),
              invm=invm, compliance=comp, side=n, ball=ball, pinned=pin)


def training_bodies(n_bodies=256, seed=0, **kw):
  """`n_bodies` seeded training bodies (`training_body`), generated one at a
  time so the set never sits in memory at once."""
  rng = np.random.default_rng(seed)
  for _ in range(int(n_bodies)):
    yield training_body(rng, **kw)
