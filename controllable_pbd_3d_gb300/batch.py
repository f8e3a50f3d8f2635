"""Many independent soft bodies in one MGPBD step.

Bodies share no vertices, so packing them into one mesh (vertex ids of body
b shifted by the vertices before it) makes the system matrix block diagonal:
one persistent-kernel CG solve fills the GPU with bodies that would each
occupy a few SMs.  Each body keeps its own compliance (alpha~ per tet).

With the FAST persistent Chebyshev CG (`per_body=True`, the default for
that mode) every body runs its own Newton loop: its residual norm, its
stopping test and its line-search step, so a stiff body does not set the
iteration count or the step of the others (`mgpbd_set_bodies`).  Each
Newton iteration solves the block-diagonal system once, and the solve is
verified per body (each active body's residual below the relative
tolerance times its own right-hand side).  A packed substep therefore
lands where separate per-body substeps land (tested).  Other modes share
one Newton loop (one residual, test and step for the whole batch).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import meshgen
from .mgpbd_gpu import MGPBDSolverGPU


@dataclass
class Body:
  x_ref: np.ndarray  # (nv, 3) float32
  x0: np.ndarray     # (nv, 3) float32
  invm: np.ndarray   # (nv,) float32
  t_i: np.ndarray    # (4 nt,) int32
  compliance: float  # XPBD compliance of its constraints


def pack_bodies(bodies):
  """Concatenate bodies into one mesh.  Returns (x_ref, x0, invm, t_i,
  vert_off, tet_off) with body b's vertices at vert_off[b]:vert_off[b+1]
  and tets at tet_off[b]:tet_off[b+1]."""
  vert_off = np.zeros(len(bodies) + 1, np.int64)
  tet_off = np.zeros(len(bodies) + 1, np.int64)
  for b, body in enumerate(bodies):
    vert_off[b + 1] = vert_off[b] + len(body.x_ref)
    tet_off[b + 1] = tet_off[b] + len(body.t_i) // 4
  if vert_off[-1] >= 2**31 or 4 * tet_off[-1] >= 2**31:
    raise OverflowError('packed mesh exceeds int32 indexing')
  x_ref = np.concatenate([b.x_ref for b in bodies]).astype(np.float32)
  x0 = np.concatenate([b.x0 for b in bodies]).astype(np.float32)
  invm = np.concatenate([b.invm for b in bodies]).astype(np.float32)
  t_i = np.concatenate([b.t_i.astype(np.int64) + vert_off[k]
                        for k, b in enumerate(bodies)]).astype(np.int32)
  return x_ref, x0, invm, t_i, vert_off, tet_off


def random_bodies(n_bodies: int, seed: int = 0, dims=(6, 30), compliance=(1e-8, 1e-5),
                  spacing: float = 0.5):
  """Hex-grid bodies with per-axis cell counts uniform in `dims`, compliance
  log-uniform in `compliance`, the top face pinned, vertices jittered by
  1 % of the cell size; bodies are laid out side by side `spacing` apart."""
  rng = np.random.default_rng(seed)
  bodies, x_shift = [], 0.0
  for _ in range(n_bodies):
    nx, ny, nz = (int(v) for v in rng.integers(dims[0], dims[1] + 1, size=3))
    h = 1.0 / 40
    xr, t = meshgen.hex_grid_tets(nx, ny, nz, h=h, origin=(x_shift, 0.0, 0.0))
    x0, _ = meshgen.hex_grid_tets(nx, ny, nz, h=h, origin=(x_shift, 0.0, 0.0), jitter=0.01,
                                  seed=int(rng.integers(2**31)))
    invm = np.ones(len(xr), np.float32)
    invm[meshgen.grid_face_vertices(nx, ny, nz, axis=1, side='max')] = 0.0
    c = float(10.0 ** rng.uniform(np.log10(compliance[0]), np.log10(compliance[1])))
    bodies.append(Body(xr.astype(np.float32), x0.astype(np.float32), invm, t.astype(np.int32), c))
    x_shift += nx * h + spacing
  return bodies


class BodyBatch:
  """One MGPBDSolverGPU over the packed bodies; `positions(b)` is a view of
  body b's rows of the shared positions tensor."""

  def __init__(self, bodies, gravity, dt, device='cuda', per_body=None, **solver_kw):
    if 'compliance' in solver_kw:
      raise ValueError('compliance is per body (Body.compliance)')
    self.bodies = list(bodies)
    xr, x0, invm, t_i, self.vert_off, self.tet_off = pack_bodies(self.bodies)
    self.x = torch.tensor(x0, device=device)
    # any positive compliance selects alpha~ = compliance / dt^2; the per-body
    # values are written after init
    self.solver = MGPBDSolverGPU(self.x, torch.tensor(xr, device=device),
                                 torch.tensor(invm, device=device),
                                 torch.tensor(t_i, device=device), None, gravity, dt,
                                 compliance=self.bodies[0].compliance, **solver_kw)
    self.dt = float(dt)
    fast_cheb = (solver_kw.get('mode') == 'fast' and solver_kw.get('precond') == 'cheb' and
                 solver_kw.get('persistent', True))
    self.per_body = fast_cheb if per_body is None else bool(per_body)
    if self.per_body:
      self.solver.set_bodies(self.vert_off, self.segments())

  def constraint_body(self) -> np.ndarray:
    """Body id of every constraint: one per tet (ARAP), or the volume
    constraints in tet order followed by the length constraints (their
    body from the edge's first vertex) with constraints='edge_volume'."""
    tet_body = np.repeat(np.arange(len(self.bodies)), np.diff(self.tet_off))
    if self.solver.constraint_kind != 'edge_volume':
      return tet_body
    edge_body = np.searchsorted(self.vert_off, self.solver.edges[:, 0], side='right') - 1
    return np.concatenate([tet_body, edge_body])

  def segments(self) -> np.ndarray:
    """(k, 3) constraint ranges (begin, end, body) in constraint order:
    each body's volume (or ARAP) constraints, then, with
    constraints='edge_volume', each body's edges (the edges are sorted by
    vertex id, so every body's edges are contiguous)."""
    cb = self.constraint_body()
    cut = np.flatnonzero(np.diff(cb)) + 1
    begin = np.concatenate([[0], cut])
    end = np.concatenate([cut, [len(cb)]])
    return np.stack([begin, end, cb[begin]], axis=1).astype(np.int32)

  def init(self):
    self.solver.init()
    comp = np.array([b.compliance for b in self.bodies], np.float64)
    alpha = (comp[self.constraint_body()] / (self.dt * self.dt)).astype(np.float32)
    self.solver.alpha_tilde.copy_(torch.from_numpy(alpha).to(self.solver.alpha_tilde.device))

  def step(self, frame: int = 0):
    self.solver.step(frame)

  def positions(self, b: int) -> torch.Tensor:
    return self.x[self.vert_off[b]:self.vert_off[b + 1]]

  @property
  def n_tets(self) -> int:
    return int(self.tet_off[-1])

  @property
  def n_constraints(self) -> int:
    return int(self.solver.n_tets)

  @property
  def n_verts(self) -> int:
    return int(self.vert_off[-1])
