// Greedy colouring (utils/graph_coloring.py:24-191) without materialising
// the adjacency sets: when node i is coloured, exactly the nodes j < i are
// coloured, so the colours to avoid are those of neighbours j < i.  A node's
// colour depends only on its neighbour set, so the result equals the
// reference's for any iteration order of its Python sets.
#include "coloring.h"

#include <stdexcept>
#include <string>

namespace mgpbd {

namespace {

void check_elems(const int32_t* elems, int32_t n_elements, int32_t k, int32_t n_vertices) {
  if (n_elements < 0 || n_vertices < 0 || k <= 0)
    throw std::invalid_argument("colouring: negative count or verts_per_element <= 0");
  if (n_elements > 0 && !elems) throw std::invalid_argument("colouring: null element array");
  const int64_t n = static_cast<int64_t>(n_elements) * k;
  for (int64_t i = 0; i < n; ++i)
    if (elems[i] < 0 || elems[i] >= n_vertices)
      throw std::invalid_argument("colouring: vertex id " + std::to_string(elems[i]) +
                                  " out of range");
}

// vertex -> elements containing it (ascending element id, an element listed
// once per occurrence of the vertex)
void vertex_elements(const int32_t* elems, int32_t n_elements, int32_t k, int32_t n_vertices,
                     std::vector<int32_t>& ptr, std::vector<int32_t>& idx) {
  ptr.assign(static_cast<size_t>(n_vertices) + 1, 0);
  const int64_t n = static_cast<int64_t>(n_elements) * k;
  for (int64_t i = 0; i < n; ++i) ptr[elems[i] + 1] += 1;
  for (int32_t v = 0; v < n_vertices; ++v) ptr[v + 1] += ptr[v];
  idx.resize(static_cast<size_t>(n));
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int32_t e = 0; e < n_elements; ++e)
    for (int32_t l = 0; l < k; ++l) idx[fill[elems[static_cast<int64_t>(e) * k + l]]++] = e;
}

// smallest colour not marked for `node` (mark[c] == node + 1 means taken)
int32_t first_free(std::vector<int32_t>& mark, int32_t node) {
  int32_t c = 0;
  while (c < static_cast<int32_t>(mark.size()) && mark[c] == node + 1) ++c;
  return c;
}

void take(std::vector<int32_t>& mark, int32_t c, int32_t node) {
  if (c >= static_cast<int32_t>(mark.size())) mark.resize(static_cast<size_t>(c) + 1, 0);
  mark[c] = node + 1;
}

Coloring pack(const std::vector<int32_t>& colors, int32_t n_colors) {
  Coloring r;
  r.n_colors = n_colors;
  r.offsets.assign(static_cast<size_t>(n_colors) + 1, 0);
  for (int32_t c : colors) r.offsets[c + 1] += 1;
  for (int32_t c = 0; c < n_colors; ++c) r.offsets[c + 1] += r.offsets[c];
  r.ordered.resize(colors.size());
  std::vector<int32_t> fill(r.offsets.begin(), r.offsets.end() - 1);
  for (size_t i = 0; i < colors.size(); ++i) r.ordered[fill[colors[i]]++] = static_cast<int32_t>(i);
  return r;
}

}  // namespace

Coloring color_elements(const int32_t* elems, int32_t n_elements, int32_t k, int32_t n_vertices) {
  check_elems(elems, n_elements, k, n_vertices);
  std::vector<int32_t> vptr, vidx;
  vertex_elements(elems, n_elements, k, n_vertices, vptr, vidx);
  std::vector<int32_t> colors(static_cast<size_t>(n_elements), -1), mark;
  int32_t n_colors = 0;
  for (int32_t e = 0; e < n_elements; ++e) {
    for (int32_t l = 0; l < k; ++l) {
      const int32_t v = elems[static_cast<int64_t>(e) * k + l];
      for (int32_t j = vptr[v]; j < vptr[v + 1]; ++j) {
        const int32_t nb = vidx[j];
        if (nb >= e) break;  // ascending: the rest are uncoloured
        take(mark, colors[nb], e);
      }
    }
    colors[e] = first_free(mark, e);
    if (colors[e] + 1 > n_colors) n_colors = colors[e] + 1;
  }
  return pack(colors, n_colors);
}

Coloring color_vertices(const int32_t* elems, int32_t n_elements, int32_t k, int32_t n_vertices) {
  check_elems(elems, n_elements, k, n_vertices);
  std::vector<int32_t> vptr, vidx;
  vertex_elements(elems, n_elements, k, n_vertices, vptr, vidx);
  std::vector<int32_t> colors(static_cast<size_t>(n_vertices), -1), mark;
  int32_t n_colors = 0;
  for (int32_t v = 0; v < n_vertices; ++v) {
    for (int32_t j = vptr[v]; j < vptr[v + 1]; ++j) {
      const int64_t e = vidx[j];
      for (int32_t l = 0; l < k; ++l) {
        const int32_t u = elems[e * k + l];
        if (u < v) take(mark, colors[u], v);
      }
    }
    colors[v] = first_free(mark, v);
    if (colors[v] + 1 > n_colors) n_colors = colors[v] + 1;
  }
  return pack(colors, n_colors);
}

Coloring greedy_coloring_csr(const int32_t* adj_ptr, const int32_t* adj, int32_t n) {
  if (n < 0) throw std::invalid_argument("colouring: negative node count");
  if (n > 0 && (!adj_ptr || (adj_ptr[n] > 0 && !adj)))
    throw std::invalid_argument("colouring: null adjacency");
  if (n > 0 && adj_ptr[0] != 0) throw std::invalid_argument("colouring: adj_ptr[0] != 0");
  for (int32_t i = 0; i < n; ++i) {
    if (adj_ptr[i + 1] < adj_ptr[i]) throw std::invalid_argument("colouring: adj_ptr decreases");
    for (int32_t j = adj_ptr[i]; j < adj_ptr[i + 1]; ++j)
      if (adj[j] < 0 || adj[j] >= n)
        throw std::invalid_argument("colouring: neighbour id out of range");
  }
  std::vector<int32_t> colors(static_cast<size_t>(n), -1), mark;
  int32_t n_colors = 0;
  for (int32_t i = 0; i < n; ++i) {
    for (int32_t j = adj_ptr[i]; j < adj_ptr[i + 1]; ++j)
      if (adj[j] < i) take(mark, colors[adj[j]], i);
    colors[i] = first_free(mark, i);
    if (colors[i] + 1 > n_colors) n_colors = colors[i] + 1;
  }
  return pack(colors, n_colors);
}

}  // namespace mgpbd
