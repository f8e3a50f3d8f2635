// Adaptive-zone kernels (zone.cu): active flags per tet (int32 0/1).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mgpbd {

// active[t] = 1 iff a vertex of t is within `radius` of (cx, cy, cz)
void launch_zone_proximity(const int32_t* t_i, const float* x, int32_t nt, float cx, float cy,
                           float cz, float radius, int32_t* active, cudaStream_t s);
// active[t] = 1 iff max over its vertices of |x - x_old| / dt > threshold
void launch_zone_strain(const int32_t* t_i, const float* x, const float* x_old, int32_t nt,
                        float threshold, float dt, int32_t* active, cudaStream_t s);
// n_rings rings of face-adjacent growth (adjacency CSR adj_ptr / adj);
// scratch holds nt int32
void launch_zone_expand(const int32_t* adj_ptr, const int32_t* adj, int32_t nt, int32_t n_rings,
                        int32_t* active, int32_t* scratch, cudaStream_t s);
// saved = alpha; alpha[t] = 1e20 where active[t] == 0
void launch_mask_alpha(const int32_t* active, float* alpha, float* saved, int32_t nt,
                       cudaStream_t s);

}  // namespace mgpbd
