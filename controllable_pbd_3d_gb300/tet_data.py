"""Tetrahedral mesh ingest with the reference's `TetData` / `load_tets`
interface (`data/tet_data.py:9-94`), on torch CUDA tensors.

`load_tets` reads a MEDIT `.mesh` file (the reference goes through meshio,
`utils/io.py:11-19`; `meshgen.parse_medit_mesh` reads the same sections, in
float64 like meshio),
keeps every other boundary triangle when `remove_duplicate` (`:88-91`),
swaps the last two indices of every triangle (`utils/geom3d.py:61-67`), and
builds the fields the solvers take: positions `v_p` / `v_p_ref` (scaled,
then shifted by `repose`), `t_i`, `f_i`, the inverse lumped vertex masses
`v_invm` and the tet volumes `t_m` (`utils/geom3d.py:48-59`), and the
surface vertex list in order of first appearance in the faces
(`extract_surface`, `data/tet_data.py:48-73`).
"""

from __future__ import annotations

import numpy as np
import torch

from .meshgen import parse_medit_mesh


def vertex_mass(verts: np.ndarray, t_i: np.ndarray):
  """(vertex order, vertex mass, tet mass): a quarter of each tet's volume
  on each of its vertices, accumulated in tet order (float64)."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  p = np.asarray(verts, np.float64)[t]
  c = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
  d = p[:, 3] - p[:, 0]
  # a batched 3-vector dot through matmul: numpy's dot kernel, the same sums
  # as the reference's per-tet np.dot
  vol = np.abs((c[:, None, :] @ d[:, :, None])[:, 0, 0]) / 6.0
  n = len(verts)
  m = np.zeros(n, np.float64)
  np.add.at(m, t.reshape(-1), np.repeat(vol / 4.0, 4))
  order = np.bincount(t.reshape(-1), minlength=n).astype(np.int64)
  return order, m, vol


def revert_faces(f_i: np.ndarray) -> np.ndarray:
  """Swap the second and third index of every triangle."""
  f = np.asarray(f_i).reshape(-1, 3).copy()
  f[:, [1, 2]] = f[:, [2, 1]]
  return f.reshape(-1)


class TetData:
  """A tet mesh on the GPU with the reference's field names."""

  def __init__(self, verts: np.ndarray, faces: np.ndarray, tets: np.ndarray, scale=1.0,
               repose=(0.0, 0.0, 0.0), device='cuda'):
    faces = np.asarray(faces)
    tets = np.asarray(tets)
    if faces.ndim != 1 or tets.ndim != 1:
      raise ValueError('faces and tets must be flat 1-D index arrays')
    self.n_verts = int(verts.shape[0])
    self.n_faces = faces.shape[0] // 3
    self.n_tets = tets.shape[0] // 4
    v64 = np.asarray(verts, np.float64) * scale + np.asarray(repose, np.float32)
    v = v64.astype(np.float32)
    self.verts_np = v64
    self.faces_np = faces.astype(np.int32)
    _, vm, tm = vertex_mass(v64, tets)
    if np.any(vm <= 0):
      raise ValueError('every vertex must belong to a tet of nonzero volume')
    self.v_p = torch.tensor(v, device=device)
    self.v_p_ref = torch.tensor(v, device=device)
    self.f_i = torch.tensor(self.faces_np, device=device)
    self.t_i = torch.tensor(tets.astype(np.int32), device=device)
    self.v_invm = torch.tensor((1.0 / vm).astype(np.float32), device=device)
    self.t_m = torch.tensor(tm.astype(np.float32), device=device)
    self.extract_surface()

  def extract_surface(self):
    """Surface vertices in order of first appearance in the faces, and the
    faces re-indexed to them."""
    f = self.faces_np
    uniq, first = np.unique(f, return_index=True)
    vert_idx = uniq[np.argsort(first, kind='stable')].astype(np.int32)
    corres = np.full(self.n_verts, -1, np.int32)
    corres[vert_idx] = np.arange(len(vert_idx), dtype=np.int32)
    self.n_surface_verts = len(vert_idx)
    dev = self.v_p.device
    self.surface_v_i = torch.tensor(vert_idx, device=dev)
    self.surface_f_i = torch.tensor(corres[f], device=dev)
    self.surface_v_p = torch.empty((self.n_surface_verts, 3), dtype=torch.float32, device=dev)
    self.update_surface_verts()

  def update_surface_verts(self):
    self.surface_v_p.copy_(self.v_p.index_select(0, self.surface_v_i.long()))


def load_tets(tetpath: str, scale=1.0, repose=(0.0, 0.0, 0.0), reverse_face=False,
              remove_duplicate=True, device='cuda') -> TetData:
  """`data/tet_data.py:80-94`: a `.mesh` file as a `TetData`."""
  if not tetpath.endswith('.mesh'):
    raise ValueError('tetpath should be a .mesh file')
  verts, tets, faces = parse_medit_mesh(tetpath, np.float64)
  if reverse_face:
    faces = faces.reshape(-1, 3)[:, ::-1].reshape(-1)
  if remove_duplicate:
    faces = faces.reshape(-1, 3)[::2].reshape(-1)
  return TetData(verts, revert_faces(faces), tets, scale, repose, device)
