"""Greedy graph colouring with the API of the reference's
`utils/graph_coloring.py:1-191`, computed by libmgpbd.so's host code
(`mgpbd_color_elements`, `mgpbd_color_vertices`, `mgpbd_greedy_coloring`).

Nodes are coloured in index order with the smallest colour no coloured
neighbour has, then grouped by colour with nodes ascending inside each
colour: the same colouring, bit for bit, as the reference's.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N


@dataclass
class ColoringResult:
  """ordered_indices: nodes grouped by colour; color_offsets[i]:[i+1] is
  colour i's range in ordered_indices; num_colors: colours used."""
  ordered_indices: np.ndarray
  color_offsets: list
  num_colors: int


_ALGORITHMS = ('greedy',)


def _check_algorithm(algorithm):
  if algorithm not in _ALGORITHMS:
    raise ValueError(f"Unknown coloring algorithm: '{algorithm}'. "
                     f"Available: {list(_ALGORITHMS)}")


def _elems(element_indices, n_elements, k):
  if hasattr(element_indices, 'to_numpy'):
    element_indices = element_indices.to_numpy()
  if hasattr(element_indices, 'detach'):
    element_indices = element_indices.detach().cpu().numpy()
  e = np.ascontiguousarray(np.asarray(element_indices).reshape(-1)[:n_elements * k], np.int32)
  if len(e) != n_elements * k:
    raise ValueError('element_indices holds fewer than n_elements * verts_per_element ids')
  return e


def _run(fn, n_nodes, *args):
  ordered = np.empty(max(n_nodes, 1), np.int32)
  offsets = np.empty(n_nodes + 1, np.int32)
  nc = C.c_int32()
  N.check(fn(*args, ordered.ctypes.data, offsets.ctypes.data, C.byref(nc)), fn.__name__)
  return ColoringResult(ordered_indices=ordered[:n_nodes].copy(),
                        color_offsets=offsets[:nc.value + 1].tolist(), num_colors=nc.value)


def build_element_adjacency(element_indices, n_elements, verts_per_element, n_vertices):
  """Elements sharing a vertex (utils/graph_coloring.py:24-49), list of sets."""
  e = _elems(element_indices, n_elements, verts_per_element).reshape(n_elements, -1)
  v2e = [[] for _ in range(n_vertices)]
  for i in range(n_elements):
    for v in e[i]:
      v2e[v].append(i)
  adj = [set() for _ in range(n_elements)]
  for i in range(n_elements):
    for v in e[i]:
      adj[i].update(v2e[v])
    adj[i].discard(i)
  return adj


def build_vertex_adjacency(element_indices, n_elements, verts_per_element, n_vertices):
  """Vertices sharing an element (utils/graph_coloring.py:52-75), list of sets."""
  e = _elems(element_indices, n_elements, verts_per_element).reshape(n_elements, -1)
  adj = [set() for _ in range(n_vertices)]
  for row in e:
    for i in range(len(row)):
      for j in range(i + 1, len(row)):
        adj[row[i]].add(int(row[j]))
        adj[row[j]].add(int(row[i]))
  return adj


def greedy_coloring(adjacency, n_nodes):
  """utils/graph_coloring.py:78-103 over a list of neighbour iterables."""
  lens = [len(adjacency[i]) for i in range(n_nodes)]
  ptr = np.zeros(n_nodes + 1, np.int32)
  ptr[1:] = np.cumsum(lens)
  adj = np.fromiter((int(j) for i in range(n_nodes) for j in adjacency[i]), np.int32,
                    count=int(ptr[-1]))
  if len(adj) == 0:
    adj = np.zeros(1, np.int32)
  return _run(N.lib().mgpbd_greedy_coloring, n_nodes, ptr.ctypes.data, adj.ctypes.data,
              int(n_nodes))


def color_edges(edge_indices, n_edges, n_vertices, algorithm='greedy'):
  """Edges sharing a vertex get different colours (:110-123)."""
  _check_algorithm(algorithm)
  return color_elements(edge_indices, n_edges, 2, n_vertices)


def color_elements(element_indices, n_elements, verts_per_element, n_vertices,
                   algorithm='greedy'):
  """Elements sharing a vertex get different colours (:126-141)."""
  _check_algorithm(algorithm)
  e = _elems(element_indices, n_elements, verts_per_element)
  return _run(N.lib().mgpbd_color_elements, n_elements, e.ctypes.data, int(n_elements),
              int(verts_per_element), int(n_vertices))


def color_vertices(element_indices, n_elements, verts_per_element, n_vertices,
                   algorithm='greedy'):
  """Vertices sharing an element get different colours (:144-159)."""
  _check_algorithm(algorithm)
  e = _elems(element_indices, n_elements, verts_per_element)
  return _run(N.lib().mgpbd_color_vertices, n_vertices, e.ctypes.data, int(n_elements),
              int(verts_per_element), int(n_vertices))
