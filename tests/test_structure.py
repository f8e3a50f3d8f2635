"""Integer structure of the system, bit-exact against the reference.

Golden: tests/golden/structure.npz, produced by running the reference's own
`cons/tet_aggregation.py` and `MGPBDSolverGPU._build_sparsity_pattern` /
`GPUMultigridSolver.setup` (make_golden.py).  Checked here: the C++ builders
in libmgpbd.so (the product path) and the oracle restatement.
"""

import hashlib

import numpy as np
import pytest

from conftest import golden
from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300 import tet_aggregation as ta
from oracle import mgpbd_oracle as orc

Z = golden('structure.npz')
CASES = sorted({k.split('/')[0] for k in Z.files})


def sha(*arrays):
  h = hashlib.sha256()
  for a in arrays:
    h.update(np.ascontiguousarray(np.asarray(a, dtype=np.int64)).tobytes())
  return h.hexdigest()


@pytest.mark.parametrize('case', CASES)
def test_pattern_bit_exact(case):
  t = Z[f'{case}/t_i']
  ip, ix = ta.sparsity_pattern(t, len(t) // 4)
  assert sha(ip, ix) == str(Z[f'{case}/pattern_sha'])
  assert int(ip[-1]) == int(Z[f'{case}/nnz'])
  if f'{case}/indices' in Z.files:
    np.testing.assert_array_equal(ix, Z[f'{case}/indices'])


@pytest.mark.parametrize('case', CASES)
def test_hierarchy_bit_exact(case):
  t = Z[f'{case}/t_i']
  nt = len(t) // 4
  Ps, sizes = ta.build_tet_hierarchy(t, Z[f'{case}/x_ref'], nt)
  assert list(sizes) == [int(s) for s in Z[f'{case}/sizes']]
  if f'{case}/agg_ids' in Z.files:
    np.testing.assert_array_equal(Ps[0].indices, Z[f'{case}/agg_ids'])
    assert Ps[0].shape == (nt, sizes[1])


@pytest.mark.parametrize('case', [c for c in CASES if f'{c}/A0_data' in Z.files])
def test_galerkin_bit_exact(case):
  t = Z[f'{case}/t_i']
  nt = len(t) // 4
  ip, ix = ta.sparsity_pattern(t, nt)
  agg = Z[f'{case}/agg_ids']
  n_agg = int(Z[f'{case}/sizes'][1])
  ci, cx, cidx, coff = ta.galerkin_structure(ip, ix, Z[f'{case}/A0_data'], agg, n_agg)
  np.testing.assert_array_equal(ci, Z[f'{case}/coarse_indptr'])
  np.testing.assert_array_equal(cx, Z[f'{case}/coarse_indices'])
  np.testing.assert_array_equal(cidx, Z[f'{case}/contrib_fine_idx'])
  np.testing.assert_array_equal(coff, Z[f'{case}/contrib_offsets'])


@pytest.mark.parametrize('case', ['box5x4x5', 'cube6', 'spot', 'ball8', 'simple_sphere'])
def test_oracle_structure_matches_golden(case):
  t = Z[f'{case}/t_i']
  nt = len(t) // 4
  ip, ix = orc.sparsity_pattern(t, nt)
  assert sha(ip, ix) == str(Z[f'{case}/pattern_sha'])
  aggs, sizes = orc.tet_hierarchy(t, nt)
  assert list(sizes) == [int(s) for s in Z[f'{case}/sizes']]
  if aggs:
    np.testing.assert_array_equal(aggs[0], Z[f'{case}/agg_ids'])
  if f'{case}/A0_data' in Z.files:
    ci, cx, cidx, coff, _ = orc.galerkin(ip, ix, Z[f'{case}/A0_data'], aggs[0], sizes[1])
    np.testing.assert_array_equal(cx, Z[f'{case}/coarse_indices'])
    np.testing.assert_array_equal(cidx, Z[f'{case}/contrib_fine_idx'])


@pytest.mark.parametrize('dims,seed,ball', [((7, 3, 9), 4, False), ((9, 9, 9), 5, True),
                                            ((16, 4, 4), 6, False), ((1, 1, 1), 0, False)])
def test_cpp_matches_oracle_on_new_meshes(dims, seed, ball):
  """Beyond the fixtures: C++ builders == oracle restatement (integer work)."""
  x, t = meshgen.hex_grid_tets(*dims, jitter=0.05, seed=seed)
  if ball:
    x = meshgen.ball_project(x)
  nt = len(t) // 4
  ip, ix = ta.sparsity_pattern(t, nt)
  ip2, ix2 = orc.sparsity_pattern(t, nt)
  np.testing.assert_array_equal(ip, ip2)
  np.testing.assert_array_equal(ix, ix2)
  Ps, sizes = ta.build_tet_hierarchy(t, x, nt)
  aggs, sizes2 = orc.tet_hierarchy(t, nt)
  assert sizes == sizes2
  if aggs:
    np.testing.assert_array_equal(Ps[0].indices, aggs[0])
    rng = np.random.default_rng(seed)
    data = rng.standard_normal(len(ix)).astype(np.float32)
    data[rng.random(len(ix)) < 0.3] = 0.0  # exact zeros exercise the dropping
    c = ta.galerkin_structure(ip, ix, data, aggs[0], sizes[1])
    o = orc.galerkin(ip, ix, data, aggs[0], sizes[1])
    for a, b in zip(c, o[:4]):
      np.testing.assert_array_equal(a, b)


def test_face_adjacency_matches_oracle():
  x, t = meshgen.hex_grid_tets(4, 3, 5, jitter=0.02, seed=1)
  nt = len(t) // 4
  a = ta.build_tet_face_adjacency(t, nt)
  b = orc.face_adjacency_sets(t, nt)
  assert all(a[i] == b[i] for i in range(nt))


def test_empty_and_degenerate_inputs():
  # no tets
  ip, ix = ta.sparsity_pattern(np.zeros(0, np.int32), 0)
  assert ip.tolist() == [0] and len(ix) == 0
  # one tet: 1x1 system, no hierarchy
  ip, ix = ta.sparsity_pattern(np.array([0, 1, 2, 3], np.int32), 1)
  assert ip.tolist() == [0, 1] and ix.tolist() == [0]
  Ps, sizes = ta.build_tet_hierarchy(np.array([0, 1, 2, 3], np.int32), None, 1)
  assert Ps == [] and sizes == [1]
  # a virtual tet level (repeated vertex ids) makes no coarsening progress
  virt = np.repeat(np.arange(500, dtype=np.int32), 4)
  agg, n_agg = ta.tet_geometry_aggregation(virt, None, 500, 8)
  assert n_agg == 500 and np.array_equal(agg, np.arange(500))


def test_negative_vertex_id_rejected():
  from controllable_pbd_3d_gb300._native import MGPBDError
  with pytest.raises(MGPBDError):
    ta.sparsity_pattern(np.array([0, 1, -2, 3], np.int32), 1)
