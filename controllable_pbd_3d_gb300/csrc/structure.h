// Host-side integer structure of the MGPBD system: the level-0 sparsity
// pattern, the tet aggregation hierarchy and the Galerkin coarse patterns
// with their contribution maps.  All of it is bit-exact with the reference
// (see structure.cpp for the file:line each function follows).
#pragma once

#include <cstdint>
#include <vector>

namespace mgpbd {

struct Csr {
  int32_t n_rows = 0;
  int32_t n_cols = 0;
  std::vector<int32_t> indptr;   // n_rows + 1
  std::vector<int32_t> indices;  // nnz
  int64_t nnz() const { return indptr.empty() ? 0 : indptr.back(); }
};

// cons/mgpbd_gpu.py:153-194: row t = sorted vertex-sharing tets, then t.
Csr build_pattern(const int32_t* t_i, int32_t nt);

// cons/tet_aggregation.py:11-127 (pass 1; pass 2 cannot trigger, every tet
// is visited by pass 1).  Returns the number of aggregates.
int32_t tet_aggregate(const int32_t* t_i, int32_t nt, int32_t max_agg_size,
                      std::vector<int32_t>& agg_ids);

// cons/tet_aggregation.py:145-211.  sizes[0] = nt; aggs[l] maps level-l
// rows to level-(l+1) rows.
void tet_hierarchy(const int32_t* t_i, int32_t nt, int32_t max_coarse,
                   int32_t max_levels, std::vector<int32_t>& sizes,
                   std::vector<std::vector<int32_t>>& aggs);

struct Galerkin {
  Csr coarse;                        // sorted columns per row (scipy tocsr)
  std::vector<int32_t> contrib_idx;  // fine nnz positions, map order
  std::vector<int32_t> contrib_off;  // coarse nnz + 1
  std::vector<int32_t> diag_pos;     // position of the diagonal per coarse row
};

// cons/mgpcg_gpu.py:43-99 for a 0/1 piecewise-constant P given by agg_ids:
// coarse pattern of (P^T A) P with scipy's csr_matmat exact-zero dropping,
// evaluated in float64 in scipy's summation order, and the contribution map.
Galerkin galerkin(const Csr& fine, const float* data, const int32_t* agg_ids,
                  int32_t n_agg);

// Same as galerkin() but without value-based dropping: the structural
// pattern of P^T S P (used for levels built by matrix-graph aggregation).
Galerkin galerkin_structural(const Csr& fine, const int32_t* agg_ids, int32_t n_agg);

// Greedy aggregation of a matrix graph (used below the tet hierarchy when
// more levels are requested).  Deterministic; visits rows in order.
int32_t graph_aggregate(const Csr& a, int32_t max_agg_size, std::vector<int32_t>& agg_ids);

// cons/tet_aggregation.py:11-37 as CSR: row t = the tets sharing a face
// with t that no third tet shares, ascending.
Csr face_adjacency(const int32_t* t_i, int32_t nt);

// vertex -> (tet, local slot) incidence, tets ascending per vertex, used for
// the deterministic scatter of dlambda into dpos.
void vertex_incidence(const int32_t* t_i, int32_t nt, int32_t nv,
                      std::vector<int32_t>& ptr, std::vector<int32_t>& ent);

}  // namespace mgpbd
