"""Seeded synthetic tetrahedral bodies (input generation only, no solver math).

The reference loads MEDIT `.mesh` files through meshio (`data/tet_data.py:81-94`,
`utils/io.py:11-19`); its experiment meshes are not shipped, so the workloads
here are regular hex grids split into 5 tetrahedra per hex, optionally
jittered or projected onto a ball.  Arrays follow the reference's field
layout: positions `(NV, 3) float32`, flat tet index array `t_i` of length
`4 * NT` (`data/tet_data.py:29-37`).
"""

from __future__ import annotations

import numpy as np

# Corner offsets (dx, dy, dz) of a unit hex, corner id = dx + 2*dy + 4*dz.
_CORNERS = np.array([[(c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1] for c in range(8)],
                    dtype=np.int64)


def _five_tet_split(parity: int):
  """Five tets of one hex; `parity` alternates so shared faces conform.

  Even hexes keep the corners with an even coordinate sum as tips of the
  four corner tets; odd hexes use the other four.  The central tet joins the
  four remaining corners.
  """
  tips = [c for c in range(8) if (_CORNERS[c].sum() % 2) == parity]
  rest = [c for c in range(8) if (_CORNERS[c].sum() % 2) != parity]
  tets = []
  for c in tips:
    nbrs = [c ^ 1, c ^ 2, c ^ 4]
    tets.append([c] + nbrs)
  tets.append(rest)
  return tets


def hex_grid_tets(nx: int, ny: int, nz: int, h: float | None = None,
                  origin=(0.0, 0.0, 0.0), jitter: float = 0.0, seed: int = 0):
  """Regular `nx x ny x nz` hex grid, 5 tets per hex, positively oriented.

  Vertex id = i + (nx+1) * (j + (ny+1) * k); y is "up".  Tets are stored
  hex-major (hex id = i + nx * (j + ny * k)), five per hex.  `jitter` is the
  uniform perturbation amplitude as a fraction of `h` (vertices move by
  U(-jitter*h, +jitter*h) per coordinate, drawn from `default_rng(seed)`).
  Returns `(x, t_i)` with `x` float32 `(NV, 3)` and `t_i` int32 `(4*NT,)`.
  """
  if h is None:
    h = 1.0 / max(nx, ny, nz)
  ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                           indexing='ij')
  # flatten with i fastest
  ii = ii.transpose(2, 1, 0).reshape(-1)
  jj = jj.transpose(2, 1, 0).reshape(-1)
  kk = kk.transpose(2, 1, 0).reshape(-1)
  x = np.stack([ii, jj, kk], axis=1).astype(np.float64) * h + np.asarray(origin, np.float64)

  split = [np.array(_five_tet_split(p), dtype=np.int64) for p in (0, 1)]
  hi, hj, hk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing='ij')
  hi = hi.transpose(2, 1, 0).reshape(-1)
  hj = hj.transpose(2, 1, 0).reshape(-1)
  hk = hk.transpose(2, 1, 0).reshape(-1)
  par = (hi + hj + hk) % 2
  # local corner ids of each tet: (n_hex, 5, 4)
  local = np.where(par[:, None, None] == 0, split[0][None], split[1][None])
  cx = hi[:, None, None] + _CORNERS[local][..., 0]
  cy = hj[:, None, None] + _CORNERS[local][..., 1]
  cz = hk[:, None, None] + _CORNERS[local][..., 2]
  vid = cx + (nx + 1) * (cy + (ny + 1) * cz)
  tets = vid.reshape(-1, 4)
  # orient positively on the unperturbed grid
  p = x[tets]
  d = np.einsum('ij,ij->i', np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
  neg = d < 0
  tets[neg, 2], tets[neg, 3] = tets[neg, 3].copy(), tets[neg, 2].copy()
  if jitter > 0.0:
    rng = np.random.default_rng(seed)
    x = x + rng.uniform(-jitter * h, jitter * h, size=x.shape)
  return x.astype(np.float32), tets.reshape(-1).astype(np.int32)


def ball_project(x: np.ndarray, center=None) -> np.ndarray:
  """Radially map a cube's vertices onto the ball that the cube encloses.

  Each point keeps its direction from the centre and is moved to radius
  `r_inf * R`, where `r_inf` is its L-infinity radius (0 at the centre, 1 on
  the cube surface) and `R` is the cube's half side.
  """
  x = np.asarray(x, np.float64)
  if center is None:
    center = 0.5 * (x.min(axis=0) + x.max(axis=0))
  d = x - center
  half = 0.5 * (x.max(axis=0) - x.min(axis=0)).max()
  linf = np.abs(d).max(axis=1)
  l2 = np.linalg.norm(d, axis=1)
  scale = np.where(l2 > 0, linf / np.where(l2 > 0, l2, 1.0), 0.0)
  return (center + d * scale[:, None]).astype(np.float32)


def face_vertices(x: np.ndarray, axis: int, side: str = 'max', tol: float = 1e-6):
  """Vertex ids on the min/max face of the bounding box along `axis`."""
  c = x[:, axis]
  ref = c.max() if side == 'max' else c.min()
  span = max(float(c.max() - c.min()), 1e-30)
  return np.nonzero(np.abs(c - ref) <= tol * span)[0].astype(np.int64)


def grid_face_vertices(nx: int, ny: int, nz: int, axis: int, side: str = 'max'):
  """Vertex ids of one face of the grid, by index (robust to jitter)."""
  ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                           indexing='ij')
  coord = [ii, jj, kk][axis]
  n = [nx, ny, nz][axis]
  sel = coord == (n if side == 'max' else 0)
  vid = ii + (nx + 1) * (jj + (ny + 1) * kk)
  return np.sort(vid[sel]).astype(np.int64)


def surface_vertices(t_i: np.ndarray) -> np.ndarray:
  """Ids of vertices on boundary faces (faces used by exactly one tet)."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  faces = np.concatenate([t[:, [1, 2, 3]], t[:, [0, 2, 3]], t[:, [0, 1, 3]], t[:, [0, 1, 2]]])
  faces.sort(axis=1)
  uniq, cnt = np.unique(faces, axis=0, return_counts=True)
  return np.unique(uniq[cnt == 1].reshape(-1))


def lumped_inverse_mass(x: np.ndarray, t_i: np.ndarray, density: float = 1.0):
  """Inverse of the lumped vertex mass (a quarter of each tet volume).

  Follows `utils/geom3d.py:48-59` (vertex mass = sum of |vol|/4 over the
  vertex's tets) as used by `data/tet_data.py:39-44`.
  """
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  p = np.asarray(x, np.float64)[t]
  vol = np.abs(np.einsum('ij,ij->i', np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]),
                         p[:, 3] - p[:, 0])) / 6.0
  m = np.zeros(len(x), np.float64)
  np.add.at(m, t.reshape(-1), np.repeat(vol * density / 4.0, 4))
  with np.errstate(divide='ignore'):
    w = np.where(m > 0, 1.0 / m, 0.0)
  return w.astype(np.float32)


def cube_body(n: int, jitter: float = 0.01, seed: int = 0, pin_top: bool = True,
              h: float | None = None):
  """The standard cube workload: n^3 hexes, unit vertex mass, top face pinned.

  Returns `(x, t_i, invm)`; pinned vertices have `invm == 0`.
  """
  x, t_i = hex_grid_tets(n, n, n, h=h, jitter=jitter, seed=seed)
  invm = np.ones(len(x), np.float32)
  if pin_top:
    invm[grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  return x, t_i, invm


def parse_medit_mesh(path: str, dtype=np.float32):
  """Minimal MEDIT `.mesh` reader: returns `(verts, tets, tris)`, 0-based,
  vertices in `dtype` (meshio, which the reference uses, gives float64).

  Replaces meshio for the reference's `load_tet` (`utils/io.py:11-19`).
  """
  with open(path) as f:
    toks = ' '.join(ln.split('#', 1)[0] for ln in f).split()
  out = {}
  i = 0
  while i < len(toks):
    key = toks[i]
    if key in ('Vertices', 'Tetrahedra', 'Triangles'):
      n = int(toks[i + 1])
      width = {'Vertices': 4, 'Tetrahedra': 5, 'Triangles': 4}[key]
      vals = toks[i + 2:i + 2 + n * width]
      arr = np.array(vals, dtype=np.float64).reshape(n, width)
      out[key] = arr
      i += 2 + n * width
    else:
      i += 1
  verts = out['Vertices'][:, :3].astype(dtype)
  tets = (out['Tetrahedra'][:, :4].astype(np.int64) - 1).reshape(-1).astype(np.int32)
  tris = (out.get('Triangles', np.zeros((0, 4)))[:, :3].astype(np.int64) - 1)
  return verts, tets, tris.reshape(-1).astype(np.int32)
