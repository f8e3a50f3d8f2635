"""The Galerkin coarse level built on the GPU (`mgpbd_device_galerkin`,
`csrc/rap.cu`) against the host build (`mgpbd_host_galerkin`, itself pinned
to scipy's RAP through the oracle in test_structure): coarse row pointers,
columns, contribution map and diagonal positions bit for bit.

The reference builds this pattern on the host (cons/mgpcg_gpu.py:30-99:
scipy's P^T A P with exact-zero dropping, then the contribution map by a
Python loop); the solver's own hierarchy build runs the device builder, so
the same comparison is repeated on the coarse levels of live solvers.

Cases: the ARAP tet matrix with its tet aggregation, the edge + volume
constraint matrix with its aggregation, a matrix whose coarse sums cancel
exactly (zero dropping at both stages of the host's order), unsorted and
repeated columns, and the structural build (data NULL) that the extra
matrix-graph levels use.
"""

import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from controllable_pbd_3d_gb300 import _native as N
from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300.tet_aggregation import (galerkin_structure,
                                                       galerkin_structure_device)
from oracle import mgpbd_oracle as MO


def assert_same(host, dev, n_agg):
  ci, cx, cidx, coff = host
  di, dx, didx, doff, ddiag = dev
  np.testing.assert_array_equal(di, ci)
  np.testing.assert_array_equal(dx, cx)
  np.testing.assert_array_equal(doff, coff)
  np.testing.assert_array_equal(didx, cidx)
  rows = np.repeat(np.arange(n_agg), np.diff(ci))
  want = np.full(n_agg, -1, np.int32)
  on = np.nonzero(cx == rows)[0]
  want[rows[on]] = on
  np.testing.assert_array_equal(ddiag, want)


def arap_matrix(n=6):
  xr, t = meshgen.hex_grid_tets(n, n, n, h=1.0 / n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, h=1.0 / n, jitter=0.03, seed=1)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  nt = len(t) // 4
  dm, _, al = MO.rest_shape(xr, t, 1e5, 1 / 300, np.float32)
  _, g = MO.constraints(x0, t, dm, np.float32)
  ip, ix = MO.sparsity_pattern(t, nt)
  a = MO.fill_A(ip, ix, t, invm, g, al, np.float32)
  aggs, sizes = MO.tet_hierarchy(t, nt)
  return ip, ix, a, aggs[0], sizes[1]


def cancelling_matrix(seed=0):
  """Block-structured matrix whose coarse entries cancel exactly: integer
  values (exact in float32 and float64) with X[I, j] = 0 for some j and
  Ac[I, J] = 0 for some J whose X are not all zero."""
  rng = np.random.default_rng(seed)
  n, n_agg = 240, 40
  agg = rng.permutation(np.repeat(np.arange(n_agg), n // n_agg)).astype(np.int32)
  A = sp.random(n, n, density=0.08, random_state=seed, format='csr')
  A.data = rng.integers(-3, 4, size=A.nnz).astype(np.float64)
  A = (A + A.T + sp.identity(n) * 20).tocsr()
  A.sort_indices()
  # make some coarse sums cancel: for a few (I, J), negate the entries so
  # that their total is zero
  rows = np.repeat(np.arange(n), np.diff(A.indptr))
  for I in range(0, n_agg, 3):
    for J in range(n_agg):
      sel = np.nonzero((agg[rows] == I) & (agg[A.indices] == J))[0]
      if len(sel) >= 2:
        A.data[sel[-1]] = -A.data[sel[:-1]].sum()
        break
  return A.indptr, A.indices, A.data.astype(np.float32), agg, n_agg


def scrambled(ip, ix, a, seed=1):
  """The same matrix with each row's entries in a random order and one
  entry per row split into two repeated columns (a non-canonical CSR)."""
  rng = np.random.default_rng(seed)
  rip, rix, ra = [0], [], []
  for i in range(len(ip) - 1):
    cols = list(ix[ip[i]:ip[i + 1]])
    vals = list(a[ip[i]:ip[i + 1]])
    half = np.float32(vals[0] / 2)
    vals[0] = np.float32(vals[0] - half)
    cols.append(cols[0])
    vals.append(half)
    p = rng.permutation(len(cols))
    rix += [cols[k] for k in p]
    ra += [vals[k] for k in p]
    rip.append(len(rix))
  return (np.array(rip, np.int32), np.array(rix, np.int32), np.array(ra, np.float32))


def test_device_galerkin_validates_before_the_gpu():
  """Argument errors are found on the host, before any CUDA call."""
  L = N.lib()
  ip = np.array([0, 1, 2], np.int32)
  ix = np.array([0, 1], np.int32)
  a = np.ones(2, np.float32)
  cn, nc = C.c_int64(0), C.c_int64(0)

  def call(ip, ix, agg, n_agg):
    return L.mgpbd_device_galerkin(len(ip) - 1, ip.ctypes.data, ix.ctypes.data, a.ctypes.data,
                                   agg.ctypes.data, n_agg, C.byref(cn), C.byref(nc), None, None,
                                   None, None, None)

  assert call(ip, ix, np.array([0, 2], np.int32), 2) == -1  # aggregate id out of range
  assert call(ip, np.array([0, 5], np.int32), np.array([0, 1], np.int32), 2) == -1
  assert call(np.array([0, 2, 1], np.int32), ix, np.array([0, 1], np.int32), 2) == -1
  assert call(ip, ix, np.array([0, 0], np.int32), 0) == -1
  assert b'n' in L.mgpbd_last_error()


@pytest.mark.gpu
def test_arap_level_bit_identical(cuda):
  ip, ix, a, agg, n_agg = arap_matrix(6)
  assert_same(galerkin_structure(ip, ix, a, agg, n_agg),
              galerkin_structure_device(ip, ix, a, agg, n_agg), n_agg)


@pytest.mark.gpu
def test_cancellation_and_noncanonical_rows_bit_identical(cuda):
  ip, ix, a, agg, n_agg = cancelling_matrix()
  host = galerkin_structure(ip, ix, a, agg, n_agg)
  # the case does drop entries: fewer coarse entries than the structural
  # pattern has
  full = galerkin_structure(ip, ix, np.ones_like(a), agg, n_agg)
  assert len(host[1]) < len(full[1])
  assert_same(host, galerkin_structure_device(ip, ix, a, agg, n_agg), n_agg)
  sip, six, sa = scrambled(ip, ix, a)
  assert_same(galerkin_structure(sip, six, sa, agg, n_agg),
              galerkin_structure_device(sip, six, sa, agg, n_agg), n_agg)


@pytest.mark.gpu
def test_structural_build_equals_positive_values(cuda):
  """data NULL keeps every touched coarse column: the host build of an
  all-positive matrix (nothing can cancel)."""
  ip, ix, a, agg, n_agg = arap_matrix(5)
  assert_same(galerkin_structure(ip, ix, np.ones_like(a), agg, n_agg),
              galerkin_structure_device(ip, ix, None, agg, n_agg), n_agg)


@pytest.mark.gpu
@pytest.mark.parametrize('n', [10, 20])
def test_solver_levels_are_built_on_the_device(cuda, n):
  """The coarse levels of a live edge + volume solver (its own hierarchy
  build) equal the host build on the solver's level-0 values, and the
  values refilled from them match the float64 Galerkin product."""
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from controllable_pbd_3d_gb300.scenarios import cube_body
  torch = cuda
  xr, x0, t, invm, compliance = cube_body(n, 0)
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], 1.0 / 300,
                     compliance=compliance, constraints='edge_volume', mode='fast',
                     precond='vcycle', max_levels=2, max_coarse=60)
  s.init()
  g = s._gpu_solver
  assert g.n_levels >= 3
  A0 = g._gpu_As[0]
  ip = A0.indptr.cpu().numpy()
  ix = A0.indices.cpu().numpy()[:A0.nnz]
  a = A0.data.cpu().numpy()[:A0.nnz]
  agg = g._agg[0].cpu().numpy()
  n_agg = g._gpu_As[1].n_rows
  ci, cx, cidx, coff = galerkin_structure(ip, ix, a, agg, n_agg)
  np.testing.assert_array_equal(g._gpu_As[1].indptr.cpu().numpy(), ci)
  np.testing.assert_array_equal(g._gpu_As[1].indices.cpu().numpy()[:len(cx)], cx)
  P = sp.csr_matrix((np.ones(len(agg)), (np.arange(len(agg)), agg)), shape=(len(agg), n_agg))
  Ac = (P.T @ sp.csr_matrix((a.astype(np.float64), ix, ip)) @ P).tocsr()
  Ac.eliminate_zeros()
  Ac.sort_indices()
  np.testing.assert_array_equal(Ac.indptr, ci)
  got = g._gpu_As[1].data.cpu().numpy()[:len(cx)].astype(np.float64)
  assert np.abs(got - Ac.data).max() <= 1e-5 * np.abs(Ac.data).max()
  # the structural level below it
  A1 = g._gpu_As[1]
  agg1 = g._agg[1].cpu().numpy()
  n2 = g._gpu_As[2].n_rows
  i1 = A1.indptr.cpu().numpy()
  x1 = A1.indices.cpu().numpy()[:A1.nnz]
  ci2, cx2, _, _ = galerkin_structure(i1, x1, np.ones(len(x1), np.float32), agg1, n2)
  np.testing.assert_array_equal(g._gpu_As[2].indptr.cpu().numpy(), ci2)
  np.testing.assert_array_equal(g._gpu_As[2].indices.cpu().numpy()[:len(cx2)], cx2)
