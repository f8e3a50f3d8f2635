"""The length + volume constraint discretisation of a tet mesh: one length
constraint per unique tet edge and one volume constraint per tet, as
4-slot constraints the MGPBD library solves with the same assembly,
multigrid and CG as the reference's one-ARAP-constraint-per-tet system
(`cons/mgpbd_gpu.py:226-247`).

* volume constraint of tet t: slots (v0, v1, v2, v3), C = det F - 1 (the
  hydrostatic constraint of `cons/deform3d.py:81-83`);
* length constraint of edge (a, b), a < b: slots (a, b, a, b),
  C = |x_a - x_b| - L0 (`cons/length.py:65-90`).

Order: the tets' volume constraints in tet order, then the edges sorted by
(a, b).  The multigrid hierarchy reuses the reference's tet aggregation
(`cons/tet_aggregation.py:145-211`): a volume constraint lies in its tet's
aggregate and a length constraint in the aggregate of the lowest-numbered
tet containing its edge.
"""

from __future__ import annotations

import numpy as np

from . import _native as N

_TET_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))


def tet_edges(t_i):
  """Unique tet edges as sorted (a, b) pairs, a < b, in lexicographic
  order, and for each the lowest-numbered tet containing it."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  nt = len(t)
  e = np.concatenate([t[:, [i, j]] for i, j in _TET_EDGES])
  e.sort(axis=1)
  owner = np.tile(np.arange(nt), len(_TET_EDGES))
  order = np.lexsort((owner, e[:, 1], e[:, 0]))
  e, owner = e[order], owner[order]
  first = np.ones(len(e), bool)
  first[1:] = np.any(e[1:] != e[:-1], axis=1)
  return e[first].astype(np.int32), owner[first].astype(np.int32)


def edge_volume_system(t_i):
  """(c_i, types, edges, edge_owner): the constraints' vertex slots (4 per
  constraint, int32), their MGPBD_CONS_* types, the edges and their
  lowest-numbered tets."""
  t = np.asarray(t_i, np.int32).reshape(-1, 4)
  edges, owner = tet_edges(t)
  c = np.concatenate([t, np.stack([edges[:, 0], edges[:, 1], edges[:, 0], edges[:, 1]], 1)])
  types = np.concatenate([np.full(len(t), N.MGPBD_CONS_VOLUME, np.int32),
                          np.full(len(edges), N.MGPBD_CONS_LENGTH, np.int32)])
  return np.ascontiguousarray(c.reshape(-1)), types, edges, owner


def edge_volume_hierarchy(t_i, max_coarse=400, max_levels=4):
  """Level-0 aggregate ids of the constraints (volume constraints first,
  then edges), from the tet aggregation of the tets; None when the tet
  hierarchy has a single level."""
  from .tet_aggregation import build_tet_hierarchy
  t = np.asarray(t_i, np.int32).reshape(-1)
  nt = len(t) // 4
  v = np.zeros((int(t.max()) + 1, 3), np.float32)  # the aggregation uses topology only
  Ps, sizes = build_tet_hierarchy(t, v, nt, max_coarse=max_coarse, max_levels=max_levels)
  if len(sizes) < 2:
    return None
  agg_t = np.asarray(Ps[0].indices, np.int64)  # one 1 per row: tet -> aggregate
  _, owner = tet_edges(t)
  return np.concatenate([agg_t, agg_t[owner]]).astype(np.int32)
