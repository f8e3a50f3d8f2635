"""Float64 restatement of the comparison solvers of the MGPBD convergence
experiments: local XPBD (`Deform3D`, cons/deform3d.py:7-288), Vertex Block
Descent (`VBDSolver`, cons/vbd.py:6-361) and the greedy colourings they run on
(utils/graph_coloring.py:24-191).

TEST INFRASTRUCTURE ONLY: imported by tests/ and the smoke check as the
checker of the CUDA path, never by the library.

Pinned by tests/golden/local.npz, which the reference's own classes produced
(tests/golden/make_golden.py under a numpy stand-in for Taichi).

Element updates within one colour touch disjoint vertices, so a colour is
evaluated as one numpy batch; that is exactly the sequential order of the
reference's per-colour loop.  The serial methods loop one element at a time.
"""

from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------------------
# greedy colouring (utils/graph_coloring.py:24-191)


def _pack(colors):
  """_pack_result (:178-191): nodes grouped by colour, ascending inside."""
  colors = np.asarray(colors, np.int64)
  n_colors = int(colors.max()) + 1 if len(colors) else 0
  ordered = np.argsort(colors, kind='stable').astype(np.int32)
  offsets = np.zeros(n_colors + 1, np.int32)
  np.add.at(offsets, colors + 1, 1)
  return ordered, np.cumsum(offsets).astype(np.int32), n_colors


def greedy(adjacency, n):
  """greedy_coloring (:78-103) over a list of neighbour iterables."""
  colors = [-1] * n
  for node in range(n):
    used = {colors[j] for j in adjacency[node] if colors[j] != -1}
    c = 0
    while c in used:
      c += 1
    colors[node] = c
  return _pack(colors)


def element_adjacency(elems, n_elements, k, n_vertices):
  """build_element_adjacency (:24-49)."""
  v2e = [[] for _ in range(n_vertices)]
  for e in range(n_elements):
    for l in range(k):
      v2e[elems[e * k + l]].append(e)
  adj = [set() for _ in range(n_elements)]
  for e in range(n_elements):
    for l in range(k):
      for nb in v2e[elems[e * k + l]]:
        if nb != e:
          adj[e].add(nb)
  return adj


def vertex_adjacency(elems, n_elements, k, n_vertices):
  """build_vertex_adjacency (:52-75)."""
  adj = [set() for _ in range(n_vertices)]
  for e in range(n_elements):
    vs = [elems[e * k + l] for l in range(k)]
    for i in range(k):
      for j in range(i + 1, k):
        adj[vs[i]].add(vs[j])
        adj[vs[j]].add(vs[i])
  return adj


def color_elements(elems, n_elements, k, n_vertices):
  return greedy(element_adjacency(elems, n_elements, k, n_vertices), n_elements)


def color_vertices(elems, n_elements, k, n_vertices):
  return greedy(vertex_adjacency(elems, n_elements, k, n_vertices), n_vertices)


# ---------------------------------------------------------------------------
# shared tet kinematics


def rest_shape(x_ref, t):
  """Dm^-1 and |det Dm| / 6 per tet, Dm's columns r_k - r_4
  (cons/vbd.py:111-124; the B of cons/deform3d.py:75)."""
  q = np.asarray(t, np.int64).reshape(-1, 4)
  r = np.asarray(x_ref, np.float64)[q]
  dm = np.stack([r[:, 0] - r[:, 3], r[:, 1] - r[:, 3], r[:, 2] - r[:, 3]], axis=2)
  return np.linalg.inv(dm), np.abs(np.linalg.det(dm)) / 6.0


def _deformation(x, q, B):
  """F = D B, D's columns x_k - x_4; batched over tets (q: (m, 4))."""
  p = x[q]
  D = np.stack([p[:, 0] - p[:, 3], p[:, 1] - p[:, 3], p[:, 2] - p[:, 3]], axis=2)
  return D @ B


def _cof(F):
  """columns f2 x f3, f3 x f1, f1 x f2 (d det F / dF)."""
  f1, f2, f3 = F[:, :, 0], F[:, :, 1], F[:, :, 2]
  return np.stack([np.cross(f2, f3), np.cross(f3, f1), np.cross(f1, f2)], axis=2)


# ---------------------------------------------------------------------------
# local XPBD (cons/deform3d.py:55-288)


def xpbd_tets(x, lh, ld, tets, q_all, B_all, invm, t_m, dt, ha, da):
  """One update of the tets `tets` (pairwise vertex-disjoint, or a single
  tet), in place on x (nv, 3), lh, ld (cons/deform3d.py:57-127)."""
  tets = np.asarray(tets, np.int64)
  q = q_all[tets]
  B = B_all[tets]
  F = _deformation(x, q, B)
  w = invm[q]                                     # (m, 4)
  CH = np.linalg.det(F) - 1.0
  gH3 = _cof(F) @ np.transpose(B, (0, 2, 1))      # columns: gradients of x1..x3
  gD3 = (2.0 * F) @ np.transpose(B, (0, 2, 1))
  gH = np.concatenate([np.transpose(gH3, (0, 2, 1)), -gH3.sum(axis=2)[:, None, :]], axis=1)
  gD = np.concatenate([np.transpose(gD3, (0, 2, 1)), -gD3.sum(axis=2)[:, None, :]], axis=1)
  SH = np.einsum('ml,mlc,mlc->m', w, gH, gH)
  SD = np.einsum('ml,mlc,mlc->m', w, gD, gD)
  SDH = np.einsum('ml,mlc,mlc->m', w, gD, gH)
  aH = ha / (dt * dt * t_m[tets])
  aD = da / (dt * dt * t_m[tets])
  CD = np.einsum('mij,mij->m', F, F) - 3.0
  lH, lD = lh[tets], ld[tets]
  dH = (SDH * (CD + aD * lD) - (CH + aH * lH) * (aD + SD)) / ((aH + SH) * (aD + SD) - SDH * SDH)
  dD = -(CD + aD * lD + SDH * dH) / (aD + SD)
  upd = w[:, :, None] * (gH * dH[:, None, None] + gD * dD[:, None, None])
  np.add.at(x, q.reshape(-1), upd.reshape(-1, 3))
  lh[tets] = lH + dH
  ld[tets] = lD + dD


class Deform3D:
  """cons/deform3d.py:7-288 in float64.  `order`: 'gauss_seidel' (index
  order, one tet at a time), 'graph_coloring' (colour by colour), or
  'default', evaluated in index order (the reference's parallel loop has no
  fixed order; it equals index order when no two tets share a vertex)."""

  def __init__(self, x, x_ref, invm, t_i, t_m, dt, hydro_alpha=0.0, devia_alpha=0.0,
               method='default', coloring=None):
    self.x = x  # (nv, 3) float64, updated in place
    self.q = np.asarray(t_i, np.int64).reshape(-1, 4)
    self.B, _ = rest_shape(x_ref, t_i)
    self.invm = np.asarray(invm, np.float64)
    self.t_m = np.asarray(t_m, np.float64)
    self.dt, self.ha, self.da = float(dt), float(hydro_alpha), float(devia_alpha)
    self.method = method
    nt = len(self.q)
    self.lh = np.zeros(nt)
    self.ld = np.zeros(nt)
    if method == 'graph_coloring':
      if coloring is not None:
        # a precomputed (ordered, offsets) schedule, for meshes where the
        # pure-Python colouring would take minutes
        self.ordered, self.offsets = (np.asarray(a) for a in coloring)
      else:
        self.ordered, self.offsets, _ = color_elements(np.asarray(t_i).tolist(), nt, 4, len(x))

  def init_rest_status(self):
    pass

  def preupdate_cons(self):
    self.lh[:] = 0.0
    self.ld[:] = 0.0

  def update_cons(self):
    args = (self.q, self.B, self.invm, self.t_m, self.dt, self.ha, self.da)
    if self.method == 'graph_coloring':
      for c in range(len(self.offsets) - 1):
        xpbd_tets(self.x, self.lh, self.ld, self.ordered[self.offsets[c]:self.offsets[c + 1]],
                  *args)
    else:
      for k in range(len(self.q)):
        xpbd_tets(self.x, self.lh, self.ld, [k], *args)


class Framework:
  """The substep of cons/framework.py:27-89: prediction of every vertex,
  preupdate_cons, `passes` x update_cons, velocity update."""

  def __init__(self, x, g, dt, damp=1.0):
    self.x = x
    self.v = np.zeros_like(x)
    self.g = np.asarray(g, np.float64)
    self.dt, self.damp = float(dt), float(damp)
    self.cons = []

  def step(self, passes):
    cache = self.x.copy()
    self.x += self.v * self.dt + self.g * self.dt * self.dt
    for c in self.cons:
      c.preupdate_cons()
    for _ in range(passes):
      for c in self.cons:
        c.update_cons()
    self.v[:] = self.damp * (self.x - cache) / self.dt


# ---------------------------------------------------------------------------
# VBD (cons/vbd.py:6-361)


class VBD:
  """cons/vbd.py in float64 (method 'serial' or 'color')."""

  def __init__(self, x, x_ref, invm, t_i, gravity, dt, damp=1.0, youngs_modulus=1e4,
               poissons_ratio=0.3, damping=0.0, n_iterations=10, rho=0.0, method='serial'):
    self.x = x
    self.nv = len(x)
    self.q = np.asarray(t_i, np.int64).reshape(-1, 4)
    self.invm = np.asarray(invm, np.float64)
    self.g = np.asarray(gravity, np.float64)
    self.dt, self.damp = float(dt), float(damp)
    E, nu = float(youngs_modulus), float(poissons_ratio)
    self.mu = E / (2.0 * (1.0 + nu))
    self.lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    self.kd = float(damping)
    self.n_iterations = int(n_iterations)
    self.rho = float(rho)
    self.method = method
    self.v = np.zeros_like(x)
    self.x_old = np.zeros_like(x)
    self.x_tilde = np.zeros_like(x)
    # vertex -> (tet, local), tets ascending (cons/vbd.py:68-96)
    flat = self.q.reshape(-1)
    order = np.argsort(flat, kind='stable')
    self.adj_tet = (order // 4).astype(np.int64)
    self.adj_loc = (order % 4).astype(np.int64)
    self.adj_off = np.concatenate([[0], np.cumsum(np.bincount(flat, minlength=self.nv))])
    if method == 'color':
      self.ordered, self.offsets, _ = color_vertices(flat.tolist(), len(self.q), 4, self.nv)
    self.Dm_inv, self.vol = rest_shape(x_ref, t_i)

  def make_prediction(self):
    self.x_old[:] = self.x
    self.x_tilde[:] = self.x + self.v * self.dt + self.g * self.dt * self.dt
    self.x[:] = self.x_tilde

  def update_vel(self):
    self.v[:] = self.damp * (self.x - self.x_old) / self.dt

  def _update(self, verts):
    """Newton step of the vertices `verts` (no two share a tet)."""
    verts = np.asarray(verts, np.int64)
    verts = verts[self.invm[verts] != 0.0]
    if len(verts) == 0:
      return
    cnt = self.adj_off[verts + 1] - self.adj_off[verts]
    owner = np.repeat(np.arange(len(verts)), cnt)
    ent = np.concatenate([np.arange(self.adj_off[v], self.adj_off[v + 1]) for v in verts])
    tet, loc = self.adj_tet[ent], self.adj_loc[ent]
    B = self.Dm_inv[tet]
    F = _deformation(self.x, self.q[tet], B)
    J = np.linalg.det(F)
    cof = _cof(F)
    P = self.mu * F + (self.lam * (J - 1.0))[:, None, None] * cof
    rows = np.concatenate([B, -B.sum(axis=1, keepdims=True)], axis=1)   # (m, 4, 3)
    b = rows[np.arange(len(tet)), loc]
    V0 = self.vol[tet]
    fe = -V0[:, None] * np.einsum('mij,mj->mi', P, b)
    qv = np.einsum('mij,mj->mi', cof, b)
    He = V0[:, None, None] * (self.mu * np.einsum('mi,mi->m', b, b)[:, None, None] * np.eye(3) +
                              self.lam * qv[:, :, None] * qv[:, None, :])
    m = len(verts)
    f = np.zeros((m, 3))
    H = np.zeros((m, 3, 3))
    np.add.at(f, owner, fe)
    np.add.at(H, owner, He)
    mh = (1.0 / self.invm[verts]) / (self.dt * self.dt)
    f += mh[:, None] * (self.x_tilde[verts] - self.x[verts])
    H += mh[:, None, None] * np.eye(3)
    if self.kd > 0.0:
      f -= (self.kd / self.dt) * (self.x[verts] - self.x_old[verts])
      H += (self.kd / self.dt) * np.eye(3)
    det = np.linalg.det(H)
    ok = np.abs(det) > 1e-10
    dx = np.zeros((m, 3))
    dx[ok] = np.linalg.solve(H[ok], f[ok][:, :, None])[:, :, 0]
    self.x[verts] += dx

  def solve(self):
    om = 1.0
    self.omegas = []
    for n in range(self.n_iterations):
      prev = self.x.copy()
      if self.method == 'serial':
        for v in range(self.nv):
          self._update([v])
      else:
        for c in range(len(self.offsets) - 1):
          self._update(self.ordered[self.offsets[c]:self.offsets[c + 1]])
      if self.rho > 0.0 and n >= 1:
        om = 2.0 / (2.0 - self.rho ** 2) if n == 1 else 4.0 / (4.0 - self.rho ** 2 * om)
        moving = self.invm > 0.0
        self.x[moving] = self.x[moving] + om * (self.x[moving] - prev[moving])
      self.omegas.append(om)

  def step(self):
    self.make_prediction()
    self.solve()
    self.update_vel()
