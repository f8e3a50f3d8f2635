"""Mesh ingest (`load_tets` / `TetData`, data/tet_data.py:9-94): a MEDIT
file written from a seeded body is read back with the reference's face
handling, lumped masses and surface extraction; the reference's own mass
and face routines (`utils/geom3d.py`, outputs in `tests/golden/geom3d_ref.npz`
from `tests/golden/make_geom_fixture.py`) pin ours bit for bit."""

import numpy as np
import pytest

from conftest import golden

from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300.tet_data import revert_faces, vertex_mass


def write_medit(path, verts, tets, tris):
  with open(path, 'w') as f:
    f.write('MeshVersionFormatted 1\nDimension 3\n')
    f.write(f'Vertices\n{len(verts)}\n')
    for v in verts:
      f.write(f'{v[0]:.9g} {v[1]:.9g} {v[2]:.9g} 0\n')
    t = tets.reshape(-1, 4) + 1
    f.write(f'Tetrahedra\n{len(t)}\n')
    for q in t:
      f.write(f'{q[0]} {q[1]} {q[2]} {q[3]} 0\n')
    tr = tris.reshape(-1, 3) + 1
    f.write(f'Triangles\n{len(tr)}\n')
    for q in tr:
      f.write(f'{q[0]} {q[1]} {q[2]} 0\n')
    f.write('End\n')


def boundary_triangles(t_i):
  """Each boundary face twice (as meshing tools that write both sides do)."""
  t = t_i.reshape(-1, 4)
  faces = np.concatenate([t[:, [1, 2, 3]], t[:, [0, 3, 2]], t[:, [0, 1, 3]], t[:, [0, 2, 1]]])
  key = np.sort(faces, axis=1)
  _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
  b = faces[cnt[inv] == 1]
  return np.stack([b, b[:, [0, 2, 1]]], axis=1).reshape(-1)


def test_vertex_mass_and_faces_match_the_reference():
  z = golden('geom3d_ref.npz')
  x, t = meshgen.hex_grid_tets(4, 3, 5, jitter=0.1, seed=3)
  x = x.astype(np.float64) * 1.7
  assert np.array_equal(x, z['x']) and np.array_equal(t, z['t'])
  order, vm, tm = vertex_mass(x, t)
  assert np.array_equal(order, z['order'])
  assert np.array_equal(vm, z['vm']) and np.array_equal(tm, z['tm'])
  f = boundary_triangles(t)
  assert np.array_equal(f, z['faces'])
  assert np.array_equal(revert_faces(f), z['reverted'])


def test_load_tets_reads_a_medit_file(tmp_path, cuda_or_cpu):
  from controllable_pbd_3d_gb300.tet_data import load_tets
  x, t = meshgen.hex_grid_tets(3, 3, 3, jitter=0.05, seed=1)
  tris = boundary_triangles(t)
  path = str(tmp_path / 'body.mesh')
  write_medit(path, x, t, tris)
  d = load_tets(path, scale=2.0, repose=(0.5, -1.0, 0.25), device=cuda_or_cpu)
  xv, _, _ = meshgen.parse_medit_mesh(path, np.float64)
  v64 = xv * 2.0 + np.array([0.5, -1.0, 0.25], np.float32)
  assert np.array_equal(d.v_p.cpu().numpy(), v64.astype(np.float32))
  assert np.array_equal(d.t_i.cpu().numpy(), t)
  _, vm, tm = vertex_mass(v64, t)
  assert np.array_equal(d.v_invm.cpu().numpy(), (1.0 / vm).astype(np.float32))
  assert np.array_equal(d.t_m.cpu().numpy(), tm.astype(np.float32))
  # every other triangle kept, second and third index swapped
  f = tris.reshape(-1, 3)[::2]
  assert np.array_equal(d.f_i.cpu().numpy().reshape(-1, 3), f[:, [0, 2, 1]])
  assert d.n_faces == len(f)
  # surface: vertices in order of first appearance, faces re-indexed
  sv = d.surface_v_i.cpu().numpy()
  seen = []
  for i in d.faces_np:
    if i not in seen:
      seen.append(i)
  assert list(sv) == seen
  assert np.array_equal(sv[d.surface_f_i.cpu().numpy()], d.faces_np)
  assert np.array_equal(d.surface_v_p.cpu().numpy(), d.v_p.cpu().numpy()[sv])


def test_load_tets_rejects_other_formats(tmp_path):
  from controllable_pbd_3d_gb300.tet_data import load_tets
  with pytest.raises(ValueError):
    load_tets(str(tmp_path / 'body.obj'), device='cpu')
