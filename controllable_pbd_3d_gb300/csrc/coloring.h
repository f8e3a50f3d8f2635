// Greedy graph colouring of mesh elements and vertices (host), the
// colourings of utils/graph_coloring.py that the comparison solvers run on:
// nodes are coloured in index order, each with the smallest colour no
// already-coloured neighbour has (greedy_coloring, :78-103), then packed by
// colour with nodes ascending inside a colour (_pack_result, :176-191).
#pragma once

#include <cstdint>
#include <vector>

namespace mgpbd {

struct Coloring {
  std::vector<int32_t> ordered;  // node ids grouped by colour
  std::vector<int32_t> offsets;  // n_colors + 1 boundaries into ordered
  int32_t n_colors = 0;
};

// Elements conflict when they share a vertex (color_elements /
// build_element_adjacency, :24-49, :126-141).  elems holds
// n_elements * verts_per_element vertex ids in [0, n_vertices).
Coloring color_elements(const int32_t* elems, int32_t n_elements, int32_t verts_per_element,
                        int32_t n_vertices);

// Vertices conflict when they share an element (color_vertices /
// build_vertex_adjacency, :52-75, :144-159).
Coloring color_vertices(const int32_t* elems, int32_t n_elements, int32_t verts_per_element,
                        int32_t n_vertices);

// greedy_coloring over an explicit adjacency in CSR form (adj_ptr: n + 1,
// adj: neighbour ids in [0, n); duplicates and self loops are ignored).
Coloring greedy_coloring_csr(const int32_t* adj_ptr, const int32_t* adj, int32_t n);

}  // namespace mgpbd
