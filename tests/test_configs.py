"""The seeded synthetic bodies have the sizes of the benchmark
configurations they stand in for: vertices, tets, unique edges and level-0
nonzeros of the 10^3 and 40^3 cubes (5 tets per hex) and of the
100 x 100 x 25 stiff-drag slab.  Host only."""

import numpy as np
import pytest

from conftest import ROOT  # noqa: F401

from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300.edge_volume import tet_edges
from controllable_pbd_3d_gb300.scenarios import drag_slab
from controllable_pbd_3d_gb300.tet_aggregation import sparsity_pattern


@pytest.mark.parametrize('n, nv, nt, ne, nnz', [
    (10, 1331, 5000, 6930, 354352),
    (40, 68921, 320000, 398520, 25926232),
])
def test_cube_sizes(n, nv, nt, ne, nnz):
  x, t = meshgen.hex_grid_tets(n, n, n)
  assert len(x) == nv and len(t) == 4 * nt
  edges, _ = tet_edges(t)
  assert len(edges) == ne
  _, ix = sparsity_pattern(t, nt)
  assert len(ix) == nnz  # one ARAP constraint per tet


def test_slab_sizes():
  s = drag_slab(100, 25, 100)
  assert len(s['x_ref']) == 265226 and len(s['t_i']) == 4 * 1250000
  edges, _ = tet_edges(s['t_i'])
  assert len(edges) == 1545225
  # one long edge (101 vertices along x) pinned, plus the dragged corner
  assert len(s['pinned']) == 101 and int((s['invm'] == 0).sum()) == 102


def test_bench_workload_is_seeded():
  """bench.py's 40^3 body: jitter and the compliance draw come from seed 0,
  so both arms and every run see the same inputs."""
  import bench as B
  xr, x0, t, invm, c = B.workload(6)
  xr2, x02, t2, invm2, c2 = B.workload(6)
  assert np.array_equal(x0, x02) and c == c2
  assert 1e-9 <= c <= 1e-4
  h = 1.0 / 6
  assert np.abs(x0 - xr).max() <= 0.01 * h + 1e-7
  assert int((invm == 0).sum()) == 7 * 7  # the top face
