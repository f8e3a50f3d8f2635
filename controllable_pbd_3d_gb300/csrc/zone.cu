// Adaptive zones around the MGPBD step (cons/adaptive_zone.py:14-91,
// cons/mgpbd_adaptive.py:17-93): per-tet active flags from a tool's
// proximity or from vertex speeds, growth by face-adjacent rings, and the
// compliance mask that makes passive tets exert no force (alpha~ = 1e20).
// Flags are int32 0/1 per tet, as the reference's `tet_active` field.
#include "zone.cuh"

#include "common.h"

namespace mgpbd {

namespace {

constexpr int kT = 256;

inline int grid_for_n(int64_t n) {
  int64_t g = (n + kT - 1) / kT;
  return static_cast<int>(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

// squared distance summed x, y, z in that order, without contraction (the
// float32 arithmetic of cons/adaptive_zone.py:46-53)
__device__ __forceinline__ float dist2(float px, float py, float pz, float cx, float cy, float cz) {
  const float dx = __fsub_rn(px, cx), dy = __fsub_rn(py, cy), dz = __fsub_rn(pz, cz);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// cons/adaptive_zone.py:40-55: active iff a vertex lies within the radius
__global__ void k_zone_proximity(const int4* __restrict__ t_i, const float* __restrict__ x,
                                 int32_t nt, float cx, float cy, float cz, float r2,
                                 int32_t* __restrict__ active) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int4 q = t_i[t];
    const int32_t v[4] = {q.x, q.y, q.z, q.w};
    int32_t a = 0;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const float* p = x + 3LL * v[l];
      if (dist2(p[0], p[1], p[2], cx, cy, cz) < r2) a = 1;
    }
    active[t] = a;
  }
}

// cons/adaptive_zone.py:57-72: active iff the fastest vertex moved faster
// than the threshold, speed = |p - p_old| / dt
__global__ void k_zone_strain(const int4* __restrict__ t_i, const float* __restrict__ x,
                              const float* __restrict__ x_old, int32_t nt, float threshold,
                              float dt, int32_t* __restrict__ active) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int4 q = t_i[t];
    const int32_t v[4] = {q.x, q.y, q.z, q.w};
    float vmax = 0.0f;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const float* p = x + 3LL * v[l];
      const float* o = x_old + 3LL * v[l];
      const float speed = __fdiv_rn(sqrtf(dist2(p[0], p[1], p[2], o[0], o[1], o[2])), dt);
      if (speed > vmax) vmax = speed;
    }
    active[t] = vmax > threshold ? 1 : 0;
  }
}

// cons/adaptive_zone.py:74-85, one ring: active if active or a face
// neighbour is
__global__ void k_zone_ring(const int32_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                            const int32_t* __restrict__ in, int32_t nt,
                            int32_t* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    int32_t a = in[t] == 1 ? 1 : 0;
    for (int32_t k = adj_ptr[t]; k < adj_ptr[t + 1] && !a; ++k) a = in[adj[k]] == 1 ? 1 : 0;
    out[t] = a ? 1 : in[t];
  }
}

// cons/mgpbd_adaptive.py:66-76: saved = alpha; alpha = 1e20 where passive
__global__ void k_mask_alpha(const int32_t* __restrict__ active, float* __restrict__ alpha,
                             float* __restrict__ saved, int32_t nt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float a = alpha[t];
    saved[t] = a;
    if (active[t] == 0) alpha[t] = 1e20f;
  }
}

}  // namespace

void launch_zone_proximity(const int32_t* t_i, const float* x, int32_t nt, float cx, float cy,
                           float cz, float radius, int32_t* active, cudaStream_t s) {
  k_zone_proximity<<<grid_for_n(nt), kT, 0, s>>>(reinterpret_cast<const int4*>(t_i), x, nt, cx,
                                                 cy, cz, radius * radius, active);
  MGPBD_CHECK_LAUNCH();
}

void launch_zone_strain(const int32_t* t_i, const float* x, const float* x_old, int32_t nt,
                        float threshold, float dt, int32_t* active, cudaStream_t s) {
  k_zone_strain<<<grid_for_n(nt), kT, 0, s>>>(reinterpret_cast<const int4*>(t_i), x, x_old, nt,
                                              threshold, dt, active);
  MGPBD_CHECK_LAUNCH();
}

void launch_zone_expand(const int32_t* adj_ptr, const int32_t* adj, int32_t nt, int32_t n_rings,
                        int32_t* active, int32_t* scratch, cudaStream_t s) {
  for (int32_t r = 0; r < n_rings; ++r) {
    k_zone_ring<<<grid_for_n(nt), kT, 0, s>>>(adj_ptr, adj, active, nt, scratch);
    MGPBD_CHECK_LAUNCH();
    MGPBD_CUDA(cudaMemcpyAsync(active, scratch, sizeof(int32_t) * nt, cudaMemcpyDeviceToDevice, s));
  }
}

void launch_mask_alpha(const int32_t* active, float* alpha, float* saved, int32_t nt,
                       cudaStream_t s) {
  k_mask_alpha<<<grid_for_n(nt), kT, 0, s>>>(active, alpha, saved, nt);
  MGPBD_CHECK_LAUNCH();
}

}  // namespace mgpbd
