// Device building blocks of the matrix-free operator A = J W J^T + alpha~
// shared by the per-phase kernels (jform.cu) and the persistent CG kernel
// (jcg.cu).
//
//   vertex phase:  u_v = w_v * sum_{(t,l): t_i[4t+l] = v} x_t g_{t,l}
//   tet phase:     (A x)_t = sum_l g_{t,l} . u_{t_i[4t+l]} + alpha~_t x_t
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mgpbd {
namespace jdev {

constexpr int kVG = 4;      // lanes per vertex in the vertex phase
constexpr int kUnroll = 6;  // entries a lane loads before its gathers

// x_t read by the vertex phase: x, z + beta p, or x * sqrt(1/diag) (Lanczos)
enum Src { kSrcX = 0, kSrcZbP = 1, kSrcSqrtD = 2 };

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide float64 sum, result valid in thread 0 (fixed pattern)
__device__ __forceinline__ double block_sum_d(double v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum_d(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum_d(v);
  __syncthreads();
  return v;
}

// Block sum of per-thread float32 partials: float32 within each warp (a
// thread holds a few terms, a warp a few dozen), float64 across the warps.
// Result valid in thread 0; fixed pattern, so every block that sums the
// same values gets the same bits.
__device__ __forceinline__ double block_sum_fd(float v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum_f(v);
  if (lane == 0) sh[wid] = static_cast<double>(v);
  __syncthreads();
  double d = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) d = warp_sum_d(d);
  __syncthreads();
  return d;
}

// Publish this block's partial; returns true in the block that finished
// last (all partials visible to it).  Never waits on other blocks.
__device__ __forceinline__ bool publish_last(double v, double* partials, uint32_t* ticket) {
  __shared__ bool last;
  v = block_sum_d(v);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = v;
    __threadfence();
    const uint32_t t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

// fixed-order sum of the partials, valid in thread 0 of the block
__device__ __forceinline__ double gather_partials(const double* partials, int n) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += __ldcg(partials + i);
  return block_sum_d(acc);
}

struct TArgs {
  const int4* t_i;
  const float4* gradC;
  const float4* u;
  const float* alpha;
  const float* dinv;
  int32_t nt;
  // constraints n4 .. nt-1 are length constraints (slots a, b, a, b): their
  // gradient n (slot 0, slot 1 is -n) in gE and (a, b) in qE, from index 0
  int32_t n4;
  const float4* gE;
  const int2* qE;
};

// g . (u_a - u_b) of length constraint t >= a.n4 (two vertices, one gradient)
__device__ __forceinline__ float jt_edge(const TArgs& a, int64_t t) {
  const int64_t e = t - a.n4;
  const int2 q = __ldg(a.qE + e);
  const float4 g = __ldg(a.gE + e);
  const float4 ua = a.u[q.x], ub = a.u[q.y];
  return (g.x * ua.x + g.y * ua.y + g.z * ua.z) - (g.x * ub.x + g.y * ub.y + g.z * ub.z);
}

// sum_l g_{t,l} . u_{v_l}
__device__ __forceinline__ float jt_core(const TArgs& a, int64_t t) {
  const int4 q = a.t_i[t];
  const float4 g0 = __ldg(a.gradC + 3 * t), g1 = __ldg(a.gradC + 3 * t + 1),
               g2 = __ldg(a.gradC + 3 * t + 2);
  const float4 u0 = a.u[q.x], u1 = a.u[q.y], u2 = a.u[q.z], u3 = a.u[q.w];
  // g_{t,0} = (g0.x, g0.y, g0.z), g_{t,1} = (g0.w, g1.x, g1.y), ...
  return (g0.x * u0.x + g0.y * u0.y + g0.z * u0.z) + (g0.w * u1.x + g1.x * u1.y + g1.y * u1.z) +
         (g1.z * u2.x + g1.w * u2.y + g2.x * u2.z) + (g2.y * u3.x + g2.z * u3.y + g2.w * u3.z);
}

// Vertex phase for one vertex group of kVG lanes: returns
// sum_{incident (t,l)} x_t g_{t,l} (reduced over the group, valid in every
// lane of it) and the vertex weight in *w.  Called by whole warps (the
// group shuffles); `valid` false gives zeros.
template <int SRC>
__device__ __forceinline__ float3 jv_group(int64_t v, bool valid, int lane,
                                           const int32_t* __restrict__ inc_ptr,
                                           const float4* __restrict__ gV,
                                           const float* __restrict__ invm,
                                           const float* __restrict__ x,
                                           const float* __restrict__ p, float beta, float* w) {
  float ax = 0.f, ay = 0.f, az = 0.f;
  const float wv = valid ? invm[v] : 0.0f;
  if (valid && wv != 0.0f) {
    const int32_t k0 = inc_ptr[v], k1 = inc_ptr[v + 1];
    // up to kUnroll entries per lane in one pass (24 incident tets per
    // vertex): all entry loads first, then all dependent x gathers, so a
    // lane keeps several requests in flight instead of one
    float4 e[kUnroll];
#pragma unroll
    for (int u2 = 0; u2 < kUnroll; ++u2) {
      const int32_t k = k0 + lane + kVG * u2;
      e[u2] = k < k1 ? __ldg(gV + k) : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    }
    float xs[kUnroll];
#pragma unroll
    for (int u2 = 0; u2 < kUnroll; ++u2) {
      const int32_t t = __float_as_int(e[u2].w);
      float xt = 0.0f;
      if (t >= 0) {
        if (SRC == kSrcZbP) xt = x[t] + beta * p[t];
        else if (SRC == kSrcSqrtD) xt = x[t] * sqrtf(p[t]);
        else xt = x[t];
      }
      xs[u2] = xt;
    }
#pragma unroll
    for (int u2 = 0; u2 < kUnroll; ++u2) {
      ax += xs[u2] * e[u2].x;
      ay += xs[u2] * e[u2].y;
      az += xs[u2] * e[u2].z;
    }
    // vertices with more than kVG * kUnroll incident tets
    for (int32_t k = k0 + lane + kVG * kUnroll; k < k1; k += kVG) {
      const float4 ee = __ldg(gV + k);
      const int32_t t = __float_as_int(ee.w);
      float xt;
      if (SRC == kSrcZbP) xt = x[t] + beta * p[t];
      else if (SRC == kSrcSqrtD) xt = x[t] * sqrtf(p[t]);
      else xt = x[t];
      ax += xt * ee.x;
      ay += xt * ee.y;
      az += xt * ee.z;
    }
  }
#pragma unroll
  for (int o = kVG / 2; o > 0; o >>= 1) {
    ax += __shfl_xor_sync(0xffffffffu, ax, o, kVG);
    ay += __shfl_xor_sync(0xffffffffu, ay, o, kVG);
    az += __shfl_xor_sync(0xffffffffu, az, o, kVG);
  }
  *w = wv;
  return make_float3(ax, ay, az);
}

}  // namespace jdev
}  // namespace mgpbd
