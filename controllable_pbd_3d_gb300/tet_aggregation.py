"""Tet aggregation hierarchy with the API of the reference's
`cons/tet_aggregation.py`, computed by the C++ builder in libmgpbd.so.

The aggregate ids are identical to the reference's, including its tie order
(the reference breaks ties by CPython set iteration order; the C++ builder
models that order exactly, see csrc/structure.cpp).  The reference's
O(NT^2) `set(np.where(visited)[0])` is replaced by O(1) membership tests, so
the 1.25M-tet slab builds in seconds instead of hours.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _native as N


def _as_i32(a):
  return np.ascontiguousarray(np.asarray(a).reshape(-1), dtype=np.int32)


def build_tet_face_adjacency(t_i_np, n_tets):
  """`cons/tet_aggregation.py:11-37`: tet -> set of tets sharing a face
  (faces shared by exactly two tets)."""
  t = _as_i32(t_i_np)[:4 * n_tets].reshape(n_tets, 4).astype(np.int64)
  faces = np.concatenate([np.sort(np.delete(t, s, axis=1), axis=1) for s in range(4)])
  owner = np.tile(np.arange(n_tets), 4)
  order = np.lexsort((owner, faces[:, 2], faces[:, 1], faces[:, 0]))
  f = faces[order]
  o = owner[order]
  same = np.all(f[1:] == f[:-1], axis=1)
  adj = {i: set() for i in range(n_tets)}
  start = 0
  n = len(f)
  brk = np.nonzero(~same)[0] + 1
  bounds = np.concatenate([[0], brk, [n]])
  for a, b in zip(bounds[:-1], bounds[1:]):
    if b - a == 2:
      x, y = int(o[a]), int(o[a + 1])
      adj[x].add(y)
      adj[y].add(x)
  del start
  return adj


def tet_geometry_aggregation(t_i_np, v_p_np, n_tets, max_agg_size=8):
  """`cons/tet_aggregation.py:40-127`; returns `(agg_ids int32, n_agg)`.

  `v_p_np` is accepted for API compatibility: the reference uses it only in
  its nearest-centroid pass, which never runs (pass 1 visits every tet).
  """
  del v_p_np
  t = _as_i32(t_i_np)
  agg = np.empty(n_tets, np.int32)
  n_agg = C.c_int32(0)
  N.check(N.lib().mgpbd_host_aggregate(t.ctypes.data, int(n_tets), int(max_agg_size),
                                       agg.ctypes.data, C.byref(n_agg)), 'mgpbd_host_aggregate')
  return agg, int(n_agg.value)


def build_prolongation_from_aggregates(agg_ids, n_tets, n_agg):
  """`cons/tet_aggregation.py:130-142`: piecewise-constant P (n_tets x n_agg)."""
  rows = np.arange(n_tets, dtype=np.int32)
  cols = np.asarray(agg_ids).astype(np.int32)
  return sp.csr_matrix((np.ones(n_tets, dtype=np.float64), (rows, cols)), shape=(n_tets, n_agg))


def build_tet_hierarchy(t_i_np, v_p_np, n_tets, max_coarse=400, max_levels=4):
  """`cons/tet_aggregation.py:145-211`: returns `(Ps, sizes)`."""
  del v_p_np
  t = _as_i32(t_i_np)
  sizes = np.zeros(max_levels + 1, np.int32)
  agg = np.empty(n_tets, np.int32)
  nl = C.c_int32(0)
  N.check(N.lib().mgpbd_host_tet_hierarchy(t.ctypes.data, int(n_tets), int(max_coarse),
                                           int(max_levels), C.byref(nl), sizes.ctypes.data,
                                           agg.ctypes.data), 'mgpbd_host_tet_hierarchy')
  sizes = [int(s) for s in sizes[:nl.value]]
  Ps = []
  if len(sizes) > 1:
    Ps.append(build_prolongation_from_aggregates(agg, n_tets, sizes[1]))
  return Ps, sizes


def sparsity_pattern(t_i_np, n_tets):
  """Level-0 CSR pattern of `cons/mgpbd_gpu.py:153-194` (diagonal last)."""
  t = _as_i32(t_i_np)
  nnz = C.c_int64(0)
  N.check(N.lib().mgpbd_host_pattern(t.ctypes.data, int(n_tets), C.byref(nnz), None, None),
          'mgpbd_host_pattern')
  indptr = np.empty(n_tets + 1, np.int32)
  indices = np.empty(nnz.value, np.int32)
  N.check(N.lib().mgpbd_host_pattern(t.ctypes.data, int(n_tets), C.byref(nnz),
                                     indptr.ctypes.data, indices.ctypes.data), 'mgpbd_host_pattern')
  return indptr, indices


def vertex_incidence(t_i_np, n_tets, n_verts):
  """Vertex-major incidence of the matrix-free operator (no reference
  counterpart): (ptr, entries) with entries 4 * t + l, ascending t, slots
  repeating an earlier vertex of their constraint left out."""
  t = _as_i32(t_i_np)
  n = C.c_int64(0)
  N.check(N.lib().mgpbd_host_vertex_incidence(t.ctypes.data, int(n_tets), int(n_verts),
                                              C.byref(n), None, None),
          'mgpbd_host_vertex_incidence')
  ptr = np.empty(n_verts + 1, np.int32)
  ent = np.empty(max(n.value, 1), np.int32)
  N.check(N.lib().mgpbd_host_vertex_incidence(t.ctypes.data, int(n_tets), int(n_verts),
                                              C.byref(n), ptr.ctypes.data, ent.ctypes.data),
          'mgpbd_host_vertex_incidence')
  return ptr, ent[:n.value]


def galerkin_structure(indptr, indices, data, agg_ids, n_agg):
  """Coarse CSR pattern and contribution map of `cons/mgpcg_gpu.py:43-99`
  for piecewise-constant P: returns (c_indptr, c_indices, contrib_idx,
  contrib_off)."""
  ip = _as_i32(indptr)
  ix = _as_i32(indices)
  d = np.ascontiguousarray(data, dtype=np.float32)
  ag = _as_i32(agg_ids)
  n = len(ip) - 1
  cn = C.c_int64(0)
  nc = C.c_int64(0)
  N.check(N.lib().mgpbd_host_galerkin(n, ip.ctypes.data, ix.ctypes.data, d.ctypes.data,
                                      ag.ctypes.data, int(n_agg), C.byref(cn), C.byref(nc),
                                      None, None, None, None), 'mgpbd_host_galerkin')
  c_indptr = np.empty(n_agg + 1, np.int32)
  c_indices = np.empty(cn.value, np.int32)
  cidx = np.empty(nc.value, np.int32)
  coff = np.empty(cn.value + 1, np.int32)
  N.check(N.lib().mgpbd_host_galerkin(n, ip.ctypes.data, ix.ctypes.data, d.ctypes.data,
                                      ag.ctypes.data, int(n_agg), C.byref(cn), C.byref(nc),
                                      c_indptr.ctypes.data, c_indices.ctypes.data,
                                      cidx.ctypes.data, coff.ctypes.data), 'mgpbd_host_galerkin')
  return c_indptr, c_indices, cidx, coff


def galerkin_structure_device(indptr, indices, data, agg_ids, n_agg):
  """The same build on the GPU (`mgpbd_device_galerkin`; bit-identical to
  `galerkin_structure`); data None gives the structural pattern.  Returns
  (c_indptr, c_indices, contrib_idx, contrib_off, diag_pos)."""
  ip = _as_i32(indptr)
  ix = _as_i32(indices)
  d = None if data is None else np.ascontiguousarray(data, dtype=np.float32)
  dp = None if d is None else d.ctypes.data
  ag = _as_i32(agg_ids)
  n = len(ip) - 1
  cn = C.c_int64(0)
  nc = C.c_int64(0)
  L = N.lib()
  N.check(L.mgpbd_device_galerkin(n, ip.ctypes.data, ix.ctypes.data, dp, ag.ctypes.data,
                                  int(n_agg), C.byref(cn), C.byref(nc), None, None, None, None,
                                  None), 'mgpbd_device_galerkin')
  c_indptr = np.empty(n_agg + 1, np.int32)
  c_indices = np.empty(max(cn.value, 1), np.int32)
  cidx = np.empty(max(nc.value, 1), np.int32)
  coff = np.empty(cn.value + 1, np.int32)
  diag = np.empty(n_agg, np.int32)
  N.check(L.mgpbd_device_galerkin(n, ip.ctypes.data, ix.ctypes.data, dp, ag.ctypes.data,
                                  int(n_agg), C.byref(cn), C.byref(nc), c_indptr.ctypes.data,
                                  c_indices.ctypes.data, cidx.ctypes.data, coff.ctypes.data,
                                  diag.ctypes.data), 'mgpbd_device_galerkin')
  return c_indptr, c_indices[:cn.value], cidx[:nc.value], coff, diag
