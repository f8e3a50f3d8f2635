// MGPBD device kernels for sm_103a.  Each kernel names the reference
// Taichi kernel whose arithmetic it reproduces.
//
// Memory layout (all in HBM, one body):
//   positions / velocities / dpos   float32 (NV, 3)      12 B/vertex
//   t_i                             int32   (NT, 4)      16 B/tet (int4 loads)
//   gradC                           float32 (NT, 4, 3)   48 B/tet (3 x float4)
//   Dm_inv                          float32 (NT, 3, 3)   36 B/tet
//   CSR level l                     int32 indptr, int32 indices, float32 data
// Reductions are float64 and deterministic: a fixed grid writes one partial
// per block, one block sums the partials in a fixed order.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>

#include "common.h"
#include "kernels.cuh"
#include "svd3.cuh"

namespace mgpbd {

std::atomic<long long> g_launches{0};

namespace {

constexpr int kThreads = 256;

inline int grid_for(int64_t work_items, int per_block) {
  int64_t g = (work_items + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > kMaxReduceBlocks) g = kMaxReduceBlocks;
  return static_cast<int>(g);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide float64 sum in a fixed pattern; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}

__device__ __forceinline__ float3 ld3(const float* p, int64_t i) {
  return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ void st3(float* p, int64_t i, float3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}

// ---------------------------------------------------------------------------
// _precompute_rest_shape (cons/mgpbd_gpu.py:136-151)
__global__ void k_rest_shape(const float* __restrict__ x_ref, const int4* __restrict__ t_i,
                             const int32_t* __restrict__ ctype, int32_t nt, float mu, float dt,
                             float* __restrict__ dm_inv, float* __restrict__ rest_vol,
                             float* __restrict__ alpha) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    int4 q = t_i[t];
    float3 r0 = ld3(x_ref, q.x), r1 = ld3(x_ref, q.y);
    if (ctype && ctype[t] == MGPBD_CONS_LENGTH) {
      // rest length of the edge (slots 0, 1); no Dm^-1
      const float dx = r0.x - r1.x, dy = r0.y - r1.y, dz = r0.z - r1.z;
      const float len = sqrtf(dx * dx + dy * dy + dz * dz);
#pragma unroll
      for (int k = 0; k < 9; ++k) dm_inv[9 * t + k] = 0.0f;
      rest_vol[t] = len;
      alpha[t] = mu < 0.0f ? (-mu) / (dt * dt) : 1.0f / (mu * dt * dt * len);
      continue;
    }
    float3 r2 = ld3(x_ref, q.z), r3 = ld3(x_ref, q.w);
    float D[3][3] = {{r1.x - r0.x, r2.x - r0.x, r3.x - r0.x},
                     {r1.y - r0.y, r2.y - r0.y, r3.y - r0.y},
                     {r1.z - r0.z, r2.z - r0.z, r3.z - r0.z}};
    float c00 = D[1][1] * D[2][2] - D[1][2] * D[2][1];
    float c01 = D[1][2] * D[2][0] - D[1][0] * D[2][2];
    float c02 = D[1][0] * D[2][1] - D[1][1] * D[2][0];
    float det = D[0][0] * c00 + D[0][1] * c01 + D[0][2] * c02;
    float inv = 1.0f / det;
    float* o = dm_inv + 9 * t;
    o[0] = c00 * inv;
    o[1] = (D[0][2] * D[2][1] - D[0][1] * D[2][2]) * inv;
    o[2] = (D[0][1] * D[1][2] - D[0][2] * D[1][1]) * inv;
    o[3] = c01 * inv;
    o[4] = (D[0][0] * D[2][2] - D[0][2] * D[2][0]) * inv;
    o[5] = (D[0][2] * D[1][0] - D[0][0] * D[1][2]) * inv;
    o[6] = c02 * inv;
    o[7] = (D[0][1] * D[2][0] - D[0][0] * D[2][1]) * inv;
    o[8] = (D[0][0] * D[1][1] - D[0][1] * D[1][0]) * inv;
    float vol = fabsf(det) / 6.0f;
    rest_vol[t] = vol;
    // mu < 0 carries a compliance: alpha~ = compliance / dt^2
    alpha[t] = mu < 0.0f ? (-mu) / (dt * dt) : 1.0f / (mu * dt * dt * vol);
  }
}

// make_prediction (cons/mgpbd_gpu.py:206-213)
__global__ void k_predict(float* __restrict__ x, float* __restrict__ v, float* __restrict__ x_old,
                          float* __restrict__ x_pred, const float* __restrict__ invm, int32_t nv,
                          float dt, float gx, float gy, float gz, float damp, int kinematic) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nv;
       k += (int64_t)gridDim.x * blockDim.x) {
    float3 p = ld3(x, k);
    float3 u = ld3(v, k);
    st3(x_old, k, p);
    if (!(kinematic && invm[k] == 0.0f)) {
      u.x = (u.x + dt * gx) * damp;
      u.y = (u.y + dt * gy) * damp;
      u.z = (u.z + dt * gz) * damp;
      p.x += dt * u.x;
      p.y += dt * u.y;
      p.z += dt * u.z;
      st3(v, k, u);
      st3(x, k, p);
    }
    if (x_pred) st3(x_pred, k, p);
  }
}

// update_vel (cons/mgpbd_gpu.py:215-219)
__global__ void k_update_vel(const float* __restrict__ x, const float* __restrict__ x_old,
                             float* __restrict__ v, int32_t nv, float dt, float damp) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nv;
       k += (int64_t)gridDim.x * blockDim.x) {
    float3 p = ld3(x, k), q = ld3(x_old, k);
    st3(v, k, make_float3(damp * (p.x - q.x) / dt, damp * (p.y - q.y) / dt, damp * (p.z - q.z) / dt));
  }
}

// F = D_s Dm^-1 for tet t at positions x (+ omega * dpos when dpos != null)
__device__ __forceinline__ void deformation(const float* __restrict__ x, const float* dpos,
                                           float omega, int4 q, const float* __restrict__ B,
                                           float (&F)[3][3]) {
  float3 p0 = ld3(x, q.x), p1 = ld3(x, q.y), p2 = ld3(x, q.z), p3 = ld3(x, q.w);
  if (dpos) {
    float3 d0 = ld3(dpos, q.x), d1 = ld3(dpos, q.y), d2 = ld3(dpos, q.z), d3 = ld3(dpos, q.w);
    p0 = make_float3(p0.x + omega * d0.x, p0.y + omega * d0.y, p0.z + omega * d0.z);
    p1 = make_float3(p1.x + omega * d1.x, p1.y + omega * d1.y, p1.z + omega * d1.z);
    p2 = make_float3(p2.x + omega * d2.x, p2.y + omega * d2.y, p2.z + omega * d2.z);
    p3 = make_float3(p3.x + omega * d3.x, p3.y + omega * d3.y, p3.z + omega * d3.z);
  }
  float Ds[3][3] = {{p1.x - p0.x, p2.x - p0.x, p3.x - p0.x},
                    {p1.y - p0.y, p2.y - p0.y, p3.y - p0.y},
                    {p1.z - p0.z, p2.z - p0.z, p3.z - p0.z}};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      F[i][j] = Ds[i][0] * B[0 * 3 + j] + Ds[i][1] * B[1 * 3 + j] + Ds[i][2] * B[2 * 3 + j];
}

__device__ __forceinline__ float arap_c(const float (&s)[3]) {
  float a = s[0] - 1.0f, b = s[1] - 1.0f, c = s[2] - 1.0f;
  return sqrtf(a * a + b * b + c * c);
}

// _compute_C_and_gradC (cons/mgpbd_gpu.py:225-247) with _arap_gradient
// (cons/mgpbd.py:35-68): G = U diag((S-1)/C) V^T Dm^-T, g0 = -(g1+g2+g3)
// Edge length constraint (cons/length.py:65-90): C = |x_a - x_b| - L0 on
// slots 0 and 1 at positions x (+ omega * dpos); gradients +-n on the two
// slots, 0 on slots 2 and 3 (which repeat the edge's vertices).
__device__ __forceinline__ float length_c(const float* __restrict__ x, const float* dpos,
                                          float omega, int4 q, float rest, float3* n) {
  float3 a = ld3(x, q.x), b = ld3(x, q.y);
  if (dpos) {
    float3 da = ld3(dpos, q.x), db = ld3(dpos, q.y);
    a = make_float3(a.x + omega * da.x, a.y + omega * da.y, a.z + omega * da.z);
    b = make_float3(b.x + omega * db.x, b.y + omega * db.y, b.z + omega * db.z);
  }
  const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  const float len = sqrtf(dx * dx + dy * dy + dz * dz);
  if (n) *n = len > 1e-12f ? make_float3(dx / len, dy / len, dz / len) : make_float3(0.f, 0.f, 0.f);
  return len - rest;
}

// Volume constraint (the hydrostatic constraint of cons/deform3d.py:81-83):
// C = det F - 1; P = d(det F)/dF = [f2 x f3, f3 x f1, f1 x f2] (columns).
__device__ __forceinline__ float volume_c(const float (&F)[3][3], float (&P)[3][3]) {
  const float f1[3] = {F[0][0], F[1][0], F[2][0]};
  const float f2[3] = {F[0][1], F[1][1], F[2][1]};
  const float f3[3] = {F[0][2], F[1][2], F[2][2]};
  const float c23[3] = {f2[1] * f3[2] - f2[2] * f3[1], f2[2] * f3[0] - f2[0] * f3[2],
                        f2[0] * f3[1] - f2[1] * f3[0]};
  const float c31[3] = {f3[1] * f1[2] - f3[2] * f1[1], f3[2] * f1[0] - f3[0] * f1[2],
                        f3[0] * f1[1] - f3[1] * f1[0]};
  const float c12[3] = {f1[1] * f2[2] - f1[2] * f2[1], f1[2] * f2[0] - f1[0] * f2[2],
                        f1[0] * f2[1] - f1[1] * f2[0]};
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    P[r][0] = c23[r];
    P[r][1] = c31[r];
    P[r][2] = c12[r];
  }
  return f1[0] * c23[0] + f1[1] * c23[1] + f1[2] * c23[2] - 1.0f;
}

__global__ void k_constraints(const float* __restrict__ x, const int4* __restrict__ t_i,
                              const int32_t* __restrict__ ctype, const float* __restrict__ dm_inv,
                              const float* __restrict__ rest, int32_t nt, float* __restrict__ C,
                              float4* __restrict__ gradC) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    int4 q = t_i[t];
    const int ty = ctype ? ctype[t] : MGPBD_CONS_ARAP;
    float g[4][3];
    if (ty == MGPBD_CONS_LENGTH) {
      float3 n;
      C[t] = length_c(x, nullptr, 0.0f, q, rest[t], &n);
      float4* o = gradC + 3 * t;
      o[0] = make_float4(n.x, n.y, n.z, -n.x);
      o[1] = make_float4(-n.y, -n.z, 0.0f, 0.0f);
      o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      continue;
    }
    float B[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) B[k] = dm_inv[9 * t + k];
    float F[3][3];
    deformation(x, nullptr, 0.0f, q, B, F);
    if (ty == MGPBD_CONS_VOLUME) {
      float P[3][3];
      C[t] = volume_c(F, P);
#pragma unroll
      for (int k = 1; k < 4; ++k)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          g[k][r] = B[(k - 1) * 3 + 0] * P[r][0] + B[(k - 1) * 3 + 1] * P[r][1] +
                    B[(k - 1) * 3 + 2] * P[r][2];
#pragma unroll
      for (int r = 0; r < 3; ++r) g[0][r] = -g[1][r] - g[2][r] - g[3][r];
      float4* o = gradC + 3 * t;
      o[0] = make_float4(g[0][0], g[0][1], g[0][2], g[1][0]);
      o[1] = make_float4(g[1][1], g[1][2], g[2][0], g[2][1]);
      o[2] = make_float4(g[2][2], g[3][0], g[3][1], g[3][2]);
      continue;
    }
    float U[3][3], s[3], V[3][3];
    svd3_rv(F, U, s, V);
    float c = arap_c(s);
    C[t] = c;
    if (c > 1e-6f) {
      float d[3] = {(s[0] - 1.0f) / c, (s[1] - 1.0f) / c, (s[2] - 1.0f) / c};
      float P[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
          P[r][cc] = U[r][0] * V[cc][0] * d[0] + U[r][1] * V[cc][1] * d[1] + U[r][2] * V[cc][2] * d[2];
#pragma unroll
      for (int k = 1; k < 4; ++k)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          g[k][r] = B[(k - 1) * 3 + 0] * P[r][0] + B[(k - 1) * 3 + 1] * P[r][1] +
                    B[(k - 1) * 3 + 2] * P[r][2];
#pragma unroll
      for (int r = 0; r < 3; ++r) g[0][r] = -g[1][r] - g[2][r] - g[3][r];
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) g[k][0] = g[k][1] = g[k][2] = 0.0f;
    }
    float4* o = gradC + 3 * t;
    o[0] = make_float4(g[0][0], g[0][1], g[0][2], g[1][0]);
    o[1] = make_float4(g[1][1], g[1][2], g[2][0], g[2][1]);
    o[2] = make_float4(g[2][2], g[3][0], g[3][1], g[3][2]);
  }
}

// _compute_rhs_gpu + _residual_norm_gpu (cons/mgpbd_gpu.py:253-267)
__global__ void k_rhs(const float* __restrict__ C, const float* __restrict__ alpha,
                      const float* __restrict__ lambda, int32_t nt, float* __restrict__ b,
                      double* __restrict__ partials) {
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    float r = -(C[t] + alpha[t] * lambda[t]);
    if (b) b[t] = r;
    acc += (double)r * (double)r;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

constexpr int kMaxOmega = 16;

// Adds constraint t's squared dual residual at x + omega_k dpos, for the
// n_omega trial steps, to acc[k] (_calc_dual_norm_at, cons/mgpbd_gpu.py:
// 360-377).
__device__ __forceinline__ void add_trials(int64_t t, const float* __restrict__ x,
                                           const float* __restrict__ dpos,
                                           const double* __restrict__ omegas, int n_omega,
                                           const int4* __restrict__ t_i,
                                           const int32_t* __restrict__ ctype,
                                           const float* __restrict__ dm_inv,
                                           const float* __restrict__ rest,
                                           const float* __restrict__ alpha,
                                           const float* __restrict__ lambda,
                                           double (&acc)[kMaxOmega]) {
  int4 q = t_i[t];
  const int ty = ctype ? ctype[t] : MGPBD_CONS_ARAP;
  float al = alpha[t] * lambda[t];
  if (ty == MGPBD_CONS_LENGTH) {
    const float L0 = rest[t];
#pragma unroll 1
    for (int k = 0; k < n_omega; ++k) {
      float r = -(length_c(x, dpos, (float)omegas[k], q, L0, nullptr) + al);
      acc[k] += (double)r * (double)r;
    }
    return;
  }
  float B[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) B[k] = dm_inv[9 * t + k];
#pragma unroll 1
  for (int k = 0; k < n_omega; ++k) {
    float F[3][3];
    deformation(x, dpos, (float)omegas[k], q, B, F);
    float c;
    if (ty == MGPBD_CONS_VOLUME) {
      float P[3][3];
      c = volume_c(F, P);
    } else {
      float U[3][3], s[3], V[3][3];
      svd3_rv(F, U, s, V);
      c = arap_c(s);
    }
    float r = -(c + al);
    acc[k] += (double)r * (double)r;
  }
}

// _calc_dual_norm_at (cons/mgpbd_gpu.py:360-377) at x + omega_k dpos for
// several omega_k in one pass
__global__ void k_dual_trial(const float* __restrict__ x, const float* __restrict__ dpos,
                             const double* __restrict__ omegas, int n_omega,
                             const int4* __restrict__ t_i, const int32_t* __restrict__ ctype,
                             const float* __restrict__ dm_inv, const float* __restrict__ rest,
                             const float* __restrict__ alpha, const float* __restrict__ lambda,
                             int32_t nt, double* __restrict__ partials) {
  double acc[kMaxOmega];
#pragma unroll
  for (int k = 0; k < kMaxOmega; ++k) acc[k] = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x)
    add_trials(t, x, dpos, omegas, n_omega, t_i, ctype, dm_inv, rest, alpha, lambda, acc);
#pragma unroll 1
  for (int k = 0; k < n_omega; ++k) {
    double v = block_sum(acc[k]);
    if (threadIdx.x == 0) partials[k * gridDim.x + blockIdx.x] = v;
  }
}

// ---------------------------------------------------------------------------
// Per-body reductions of a packed batch.  The constraints are cut into
// chunks (contiguous ranges, each inside one body's range); block c sums
// its chunk in a fixed order, so the per-body sums the host forms from the
// chunk partials (in chunk order) repeat bit for bit.

// partials[c] = sum over chunk c of (C + alpha lambda)^2 (alpha = null: C^2)
__global__ void k_chunk_dual_sq(const float* __restrict__ C, const float* __restrict__ alpha,
                                const float* __restrict__ lambda,
                                const int2* __restrict__ chunks, double* __restrict__ partials) {
  const int2 ch = chunks[blockIdx.x];
  double acc = 0.0;
  for (int64_t t = ch.x + threadIdx.x; t < ch.y; t += blockDim.x) {
    float r = alpha ? C[t] + alpha[t] * lambda[t] : C[t];
    acc += (double)r * (double)r;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// partials[k * n_chunks + c]: the dual residual squares of chunk c at the
// trial step omega_k
__global__ void k_chunk_trial(const float* __restrict__ x, const float* __restrict__ dpos,
                              const double* __restrict__ omegas, int n_omega,
                              const int4* __restrict__ t_i, const int32_t* __restrict__ ctype,
                              const float* __restrict__ dm_inv, const float* __restrict__ rest,
                              const float* __restrict__ alpha, const float* __restrict__ lambda,
                              const int2* __restrict__ chunks, double* __restrict__ partials) {
  double acc[kMaxOmega];
#pragma unroll
  for (int k = 0; k < kMaxOmega; ++k) acc[k] = 0.0;
  const int2 ch = chunks[blockIdx.x];
  for (int64_t t = ch.x + threadIdx.x; t < ch.y; t += blockDim.x)
    add_trials(t, x, dpos, omegas, n_omega, t_i, ctype, dm_inv, rest, alpha, lambda, acc);
#pragma unroll 1
  for (int k = 0; k < n_omega; ++k) {
    double v = block_sum(acc[k]);
    if (threadIdx.x == 0) partials[k * gridDim.x + blockIdx.x] = v;
  }
}

// b_t = 0 for the constraints of bodies whose Newton loop has ended
__global__ void k_mask_rhs(float* __restrict__ b, const int32_t* __restrict__ cons_body,
                           const int32_t* __restrict__ active, int32_t nt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x)
    if (!active[cons_body[t]]) b[t] = 0.0f;
}

// _apply_dpos with each body's own line-search step
__global__ void k_apply_bodies(float* __restrict__ x, const float* __restrict__ dpos,
                               const float* __restrict__ invm,
                               const int32_t* __restrict__ vert_body,
                               const float* __restrict__ omega, int32_t nv) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nv;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (invm[k] > 0.0f) {
      const float w = omega[vert_body[k]];
      float3 p = ld3(x, k), d = ld3(dpos, k);
      st3(x, k, make_float3(p.x + w * d.x, p.y + w * d.y, p.z + w * d.z));
    }
  }
}

__global__ void k_lambda_update(float* __restrict__ lambda, const float* __restrict__ dlam,
                                int32_t nt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x)
    lambda[t] += dlam[t];
}

// _zero_dpos + _scatter_dlam_gpu (cons/mgpbd_gpu.py:330-355): gathered per
// vertex over its incident (tet, slot) pairs in ascending tet order, so the
// float32 sum has the order of a serial run of the reference loop.
// With dlam_lo (the low part of a float-pair solution) the sum runs in
// float64 over dlam + dlam_lo: on stiff bodies dpos is a small difference
// of large terms w dlam g, whose float32 rounding would otherwise reach the
// 1e-5 level in positions.
__global__ void k_scatter(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc_ent,
                          const float* __restrict__ invm, const float* __restrict__ dlam,
                          const float* __restrict__ dlam_lo, const float* __restrict__ gradC,
                          float* __restrict__ dpos, int32_t nv) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x) {
    float w = invm[v];
    if (dlam_lo) {
      double ax = 0.0, ay = 0.0, az = 0.0;
      for (int32_t k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
        int32_t e = inc_ent[k];  // 4 * tet + slot
        const double sc = (double)w * ((double)dlam[e >> 2] + (double)dlam_lo[e >> 2]);
        const float* g = gradC + 3 * (int64_t)e;
        ax += sc * (double)g[0];
        ay += sc * (double)g[1];
        az += sc * (double)g[2];
      }
      st3(dpos, v, make_float3((float)ax, (float)ay, (float)az));
      continue;
    }
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    for (int32_t k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      int32_t e = inc_ent[k];  // 4 * tet + slot
      float sc = w * dlam[e >> 2];
      const float* g = gradC + 3 * (int64_t)e;
      acc.x += sc * g[0];
      acc.y += sc * g[1];
      acc.z += sc * g[2];
    }
    st3(dpos, v, acc);
  }
}

// _apply_dpos (cons/mgpbd_gpu.py:345-349)
__global__ void k_apply(float* __restrict__ x, const float* __restrict__ dpos,
                        const float* __restrict__ invm, int32_t nv, float omega) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nv;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (invm[k] > 0.0f) {
      float3 p = ld3(x, k), d = ld3(dpos, k);
      st3(x, k, make_float3(p.x + omega * d.x, p.y + omega * d.y, p.z + omega * d.z));
    }
  }
}

// ---------------------------------------------------------------------------
// _fill_A_kernel (cons/mgpbd_gpu.py:273-309) with _intersect_tets
// (cons/mgpbd.py:72-84): one warp per row of the diagonal-last pattern.
__global__ void k_fill_A(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                         const int4* __restrict__ t_i, const float* __restrict__ invm,
                         const float4* __restrict__ gradC, const float* __restrict__ alpha,
                         int32_t nt, float* __restrict__ data, float* __restrict__ diag_inv) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < nt; i += warps) {
    int4 qi = t_i[i];
    int vi[4] = {qi.x, qi.y, qi.z, qi.w};
    float4 a0 = gradC[3 * i], a1 = gradC[3 * i + 1], a2 = gradC[3 * i + 2];
    float gi[4][3] = {{a0.x, a0.y, a0.z}, {a0.w, a1.x, a1.y}, {a1.z, a1.w, a2.x}, {a2.y, a2.z, a2.w}};
    float wi[4] = {invm[vi[0]], invm[vi[1]], invm[vi[2]], invm[vi[3]]};
    int32_t k0 = indptr[i], k1 = indptr[i + 1];
    for (int32_t k = k0 + lane; k < k1 - 1; k += 32) {
      int32_t j = indices[k];
      int4 qj = t_i[j];
      int vj[4] = {qj.x, qj.y, qj.z, qj.w};
      float4 b0 = gradC[3 * (int64_t)j], b1 = gradC[3 * (int64_t)j + 1], b2 = gradC[3 * (int64_t)j + 2];
      float gj[4][3] = {{b0.x, b0.y, b0.z}, {b0.w, b1.x, b1.y}, {b1.z, b1.w, b2.x}, {b2.y, b2.z, b2.w}};
      float off = 0.0f;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if (vi[a] == vj[b])
            off += wi[a] * (gi[a][0] * gj[b][0] + gi[a][1] * gj[b][1] + gi[a][2] * gj[b][2]);
      data[k] = off;
    }
    if (lane == 0) {
      float d = 0.0f;
#pragma unroll
      for (int a = 0; a < 4; ++a)
        d += wi[a] * (gi[a][0] * gi[a][0] + gi[a][1] * gi[a][1] + gi[a][2] * gi[a][2]);
      d += alpha[i];
      data[k1 - 1] = d;
      diag_inv[i] = fabsf(d) > 1e-30f ? 1.0f / d : 0.0f;
    }
  }
}

// _fill_coarse_values_kernel (cons/mgpcg_gpu.py:183-198)
__global__ void k_rap_refill(const int32_t* __restrict__ off, const int32_t* __restrict__ idx,
                             const float* __restrict__ fine, int64_t nnz_c,
                             float* __restrict__ coarse) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nnz_c;
       c += (int64_t)gridDim.x * blockDim.x) {
    float v = 0.0f;
    for (int32_t k = off[c]; k < off[c + 1]; ++k) v += fine[idx[k]];
    coarse[c] = v;
  }
}

__global__ void k_diag_inv_pos(const int32_t* __restrict__ pos, const float* __restrict__ data,
                               int32_t n, float* __restrict__ dinv) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float d = pos[i] >= 0 ? data[pos[i]] : 0.0f;
    dinv[i] = fabsf(d) > 1e-30f ? 1.0f / d : 0.0f;
  }
}

// cache_diag_inv (cons/sparse_gpu.py:107-121)
__global__ void k_diag_inv_scan(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                const float* __restrict__ data, int32_t n, float* __restrict__ dinv) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float d = 0.0f;
    for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k)
      if (indices[k] == i) {
        d = data[k];
        break;
      }
    dinv[i] = fabsf(d) > 1e-30f ? 1.0f / d : 0.0f;
  }
}

// ---------------------------------------------------------------------------
// Row operators on CSR: G lanes per row, rows strided over a fixed grid.
enum RowOp { kSpmv = 0, kJacobi = 1, kResidual = 2, kSpmvDot = 3, kJacobiZero = 4 };

template <int G, int OP>
__global__ void __launch_bounds__(kThreads)
    k_csr_rows(int32_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
               const float* __restrict__ data, const float* __restrict__ x,
               const float* __restrict__ b, const float* __restrict__ dinv, float* __restrict__ y,
               float w, const float* __restrict__ wp, double* __restrict__ partials,
               const CgState* __restrict__ st) {
  if (st && st->done) return;
  if (wp) w = *wp;
  // The loop bound is uniform per warp (all 32/G rows of a warp advance
  // together), so every lane reaches the shuffles.
  const int lane = threadIdx.x % G;
  constexpr int kRowsPerWarp = 32 / G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t stride = ((int64_t)gridDim.x * blockDim.x >> 5) * kRowsPerWarp;
  double dacc = 0.0;
  for (int64_t base = warp * kRowsPerWarp; base < n; base += stride) {
    const int64_t row = base + (threadIdx.x & 31) / G;
    const bool valid = row < n;
    float sum = 0.0f;
    if (OP != kJacobiZero) {
      if (valid) {
        int32_t k0 = indptr[row], k1 = indptr[row + 1];
        for (int32_t k = k0 + lane; k < k1; k += G) sum += data[k] * __ldg(x + indices[k]);
      }
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, G);
    }
    if (valid && lane == 0) {
      if (OP == kSpmv) {
        y[row] = sum;
      } else if (OP == kSpmvDot) {
        y[row] = sum;
        dacc += (double)x[row] * (double)sum;
      } else if (OP == kResidual) {
        y[row] = b[row] - sum;
      } else if (OP == kJacobi) {
        y[row] = x[row] + w * dinv[row] * (b[row] - sum);
      } else {  // x = 0: A x = 0 exactly for finite A
        y[row] = w * dinv[row] * b[row];
      }
    }
  }
  if (OP == kSpmvDot) {
    dacc = block_sum(dacc);
    if (threadIdx.x == 0) partials[blockIdx.x] = dacc;
  }
}

// Vectorised variant for the library's own (padded) CSR arrays: each of the
// G lanes of a row loads U float4 values and U int4 column ids per pass from
// the 16-byte aligned window that starts at indptr[row] rounded down to a
// multiple of 4, and masks the elements outside [indptr[row], indptr[row+1]).
// The arrays carry >= 4 padding elements, so the last window stays inside
// the allocation.  All U loads of a pass are issued before the first use,
// which keeps 2*U*16 bytes per lane in flight.
template <int G, int U, int OP>
__global__ void __launch_bounds__(kThreads)
    k_csr_rows_vec(int32_t n, const int32_t* __restrict__ indptr,
                   const int32_t* __restrict__ indices, const float* __restrict__ data,
                   const float* __restrict__ x, const float* __restrict__ b,
                   const float* __restrict__ dinv, float* __restrict__ y, float w,
                   const float* __restrict__ wp, double* __restrict__ partials,
                   const CgState* __restrict__ st) {
  if (st && st->done) return;
  if (wp) w = *wp;
  const int lane = threadIdx.x % G;
  constexpr int kRowsPerWarp = 32 / G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t stride = ((int64_t)gridDim.x * blockDim.x >> 5) * kRowsPerWarp;
  double dacc = 0.0;
  for (int64_t base = warp * kRowsPerWarp; base < n; base += stride) {
    const int64_t row = base + (threadIdx.x & 31) / G;
    const bool valid = row < n;
    float sum = 0.0f;
    if (valid) {
      const int32_t k0 = indptr[row], k1 = indptr[row + 1];
      for (int32_t kb = k0 & ~3; kb < k1; kb += 4 * G * U) {
        float4 dv[U];
        int4 iv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int32_t kk = kb + 4 * (lane + G * u);
          if (kk < k1) {
            dv[u] = __ldg(reinterpret_cast<const float4*>(data + kk));
            iv[u] = __ldg(reinterpret_cast<const int4*>(indices + kk));
          } else {
            dv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            iv[u] = make_int4(0, 0, 0, 0);
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int32_t kk = kb + 4 * (lane + G * u);
          if (kk + 0 >= k0 && kk + 0 < k1) sum += dv[u].x * __ldg(x + iv[u].x);
          if (kk + 1 >= k0 && kk + 1 < k1) sum += dv[u].y * __ldg(x + iv[u].y);
          if (kk + 2 >= k0 && kk + 2 < k1) sum += dv[u].z * __ldg(x + iv[u].z);
          if (kk + 3 >= k0 && kk + 3 < k1) sum += dv[u].w * __ldg(x + iv[u].w);
        }
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, G);
    if (valid && lane == 0) {
      if (OP == kSpmv) {
        y[row] = sum;
      } else if (OP == kSpmvDot) {
        y[row] = sum;
        dacc += (double)x[row] * (double)sum;
      } else if (OP == kResidual) {
        y[row] = b[row] - sum;
      } else {
        y[row] = x[row] + w * dinv[row] * (b[row] - sum);
      }
    }
  }
  if (OP == kSpmvDot) {
    dacc = block_sum(dacc);
    if (threadIdx.x == 0) partials[blockIdx.x] = dacc;
  }
}

// Tile shapes of the vectorised row kernel: G lanes per row, each loading U
// float4 (value) + int4 (column) pairs per pass, so one pass covers 4*G*U
// nonzeros of a row.  Index 0 is the default for long rows (4 x 6: the
// ~81-nonzero rows of the level-0 ARAP matrix, SpMV 5.0 TB/s on GB300 at
// 40^3 against 4.3 for 8 x 4 and 4.8 for 4 x 8), index 1 for shorter rows;
// tune_row_shape picks among all of them by timing.
constexpr int kRowShapeG[kNumRowShapes] = {4, 4, 4, 2, 2, 4, 8, 8};
constexpr int kRowShapeU[kNumRowShapes] = {6, 4, 8, 4, 8, 2, 2, 4};

template <int OP>
void launch_vec_shape(int idx, const CsrView& a, const float* x, const float* b, float* y,
                      float w, double* partials, const CgState* st, cudaStream_t s,
                      const float* wp) {
  const int G = kRowShapeG[idx];
  const int grid = OP == kSpmvDot ? reduce_blocks(a.n) : grid_for(a.n, kThreads / G);
  switch (idx) {
#define MGPBD_VEC_CASE(I, GG, UU)                                                            \
  case I:                                                                                    \
    k_csr_rows_vec<GG, UU, OP><<<grid, kThreads, 0, s>>>(a.n, a.indptr, a.indices, a.data, x, \
                                                         b, a.diag_inv, y, w, wp, partials, st); \
    break;
    MGPBD_VEC_CASE(0, 4, 6)
    MGPBD_VEC_CASE(1, 4, 4)
    MGPBD_VEC_CASE(2, 4, 8)
    MGPBD_VEC_CASE(3, 2, 4)
    MGPBD_VEC_CASE(4, 2, 8)
    MGPBD_VEC_CASE(5, 4, 2)
    MGPBD_VEC_CASE(6, 8, 2)
    MGPBD_VEC_CASE(7, 8, 4)
#undef MGPBD_VEC_CASE
    default:
      throw Error(MGPBD_EINVAL, "unknown row-kernel shape");
  }
  MGPBD_CHECK_LAUNCH();
}

template <int OP>
void rows_dispatch(const CsrView& a, const float* x, const float* b, float* y, float w,
                   double* partials, const CgState* st, cudaStream_t s, const float* wp = nullptr) {
  if (a.n <= 0) return;
  double avg = a.n ? (double)a.nnz / a.n : 0.0;
  if (a.padded && OP != kJacobiZero) {
    const int idx = a.shape >= 0 ? a.shape : (avg >= 40 ? 0 : 1);
    launch_vec_shape<OP>(idx, a, x, b, y, w, partials, st, s, wp);
    return;
  }
  int G = avg >= 48 ? 32 : (avg >= 20 ? 16 : (avg >= 8 ? 8 : 4));
  if (OP == kJacobiZero) G = 1;
  int rows_per_block = kThreads / G;
  int grid = grid_for(a.n, rows_per_block);
  if (OP == kSpmvDot) grid = reduce_blocks(a.n);
  switch (G) {
#define MGPBD_ROWS_CASE(GG)                                                                  \
  case GG:                                                                                   \
    k_csr_rows<GG, OP><<<grid, kThreads, 0, s>>>(a.n, a.indptr, a.indices, a.data, x, b,     \
                                                 a.diag_inv, y, w, wp, partials, st);        \
    break;
    MGPBD_ROWS_CASE(1)
    MGPBD_ROWS_CASE(4)
    MGPBD_ROWS_CASE(8)
    MGPBD_ROWS_CASE(16)
    MGPBD_ROWS_CASE(32)
#undef MGPBD_ROWS_CASE
  }
  MGPBD_CHECK_LAUNCH();
}

// P^T r for piecewise-constant P: sum of the members of each aggregate in
// ascending row order (the order of the reference's P^T CSR spmv).
__global__ void k_restrict(const int32_t* __restrict__ mem_ptr, const int32_t* __restrict__ mem_rows,
                           const float* __restrict__ r, int32_t nc, float* __restrict__ bc,
                           const CgState* __restrict__ st) {
  if (st && st->done) return;
  for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < nc;
       I += (int64_t)gridDim.x * blockDim.x) {
    float v = 0.0f;
    for (int32_t k = mem_ptr[I]; k < mem_ptr[I + 1]; ++k) v += r[mem_rows[k]];
    bc[I] = v;
  }
}

// x += P xc (the reference's P spmv into tmp followed by axpy with 1.0)
__global__ void k_prolong_add(const int32_t* __restrict__ agg, const float* __restrict__ xc,
                              int32_t n, float* __restrict__ x, const CgState* __restrict__ st) {
  if (st && st->done) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += xc[agg[i]];
}

// ---------------------------------------------------------------------------
__global__ void k_dot(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                      double* __restrict__ partials, const CgState* __restrict__ st) {
  if (st && st->done) return;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)a[i] * (double)b[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void k_axpy(float alpha, const float* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += alpha * x[i];
}

__global__ void k_scale(float alpha, float* __restrict__ x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= alpha;
}

__global__ void k_xpay(float alpha, const float* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i] + alpha * y[i];
}

__device__ double sum_partials(const double* __restrict__ p, int blocks) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < blocks; i += blockDim.x) acc += p[i];
  return block_sum(acc);
}

__global__ void k_finalize(const double* __restrict__ partials, int blocks, int count,
                           double* __restrict__ out) {
  for (int g = 0; g < count; ++g) {
    double v = sum_partials(partials + (int64_t)g * blocks, blocks);
    if (threadIdx.x == 0) out[g] = v;
  }
}

// ---------------------------------------------------------------------------
// CG scalar steps (GPUMultigridSolver.solve, cons/mgpcg_gpu.py:261-329)
__global__ void k_cg_init(CgState* st, const double* __restrict__ p, int blocks, double tol_abs,
                          double tol_rel, int maxiter) {
  double rz = sum_partials(p, blocks);
  double rr0 = sum_partials(p + blocks, blocks);
  if (threadIdx.x == 0) {
    st->rz = rz;
    st->rr0 = rr0;
    double t2 = tol_abs * tol_abs;
    double r2 = tol_rel * tol_rel * rr0;
    st->tol2 = r2 > t2 ? r2 : t2;
    st->iters = 0;
    st->done = maxiter <= 0;
    st->status = isfinite(rz) ? 0 : MGPBD_STATUS_NAN;
    st->maxiter = maxiter;
    st->body_runs = 0;
    st->alpha = st->beta = st->pap = st->rr = st->rz_new = 0.0;
  }
}

__global__ void k_cg_alpha(CgState* st, const double* __restrict__ p, int blocks) {
  if (st->done) return;
  double pap = sum_partials(p, blocks);
  if (threadIdx.x == 0) {
    st->pap = pap;
    if (!isfinite(pap)) st->status |= MGPBD_STATUS_NAN;
    if (fabs(pap) < 1e-30 || !isfinite(pap)) {
      st->done = 1;
    } else {
      if (pap <= 0.0) st->status |= MGPBD_STATUS_PAP_NONPOS;
      st->alpha = st->rz / pap;
    }
  }
}

__global__ void k_cg_update_xr(const CgState* __restrict__ st, const float* __restrict__ p,
                               const float* __restrict__ ap, float* __restrict__ x,
                               float* __restrict__ r, int64_t n, double* __restrict__ partials) {
  if (st->done) return;
  float a = (float)st->alpha;
  float na = (float)(-st->alpha);
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    float ri = r[i] + na * ap[i];
    r[i] = ri;
    acc += (double)ri * (double)ri;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void k_cg_check(CgState* st, const double* __restrict__ p, int blocks) {
  if (st->done) return;
  double rr = sum_partials(p, blocks);
  if (threadIdx.x == 0) {
    st->rr = rr;
    if (!isfinite(rr)) {
      st->status |= MGPBD_STATUS_NAN;
      st->done = 1;
    } else if (rr < st->tol2) {
      st->iters += 1;
      st->done = 1;
    }
  }
}

__global__ void k_cg_beta(CgState* st, const double* __restrict__ p, int blocks) {
  if (st->done) return;
  double rzn = sum_partials(p, blocks);
  if (threadIdx.x == 0) {
    st->rz_new = rzn;
    if (fabs(st->rz) < 1e-30) {
      st->iters += 1;
      st->done = 1;
      return;
    }
    st->beta = rzn / st->rz;
    st->rz = rzn;
    st->iters += 1;
    if (st->iters >= st->maxiter) {
      st->done = 1;
      st->status |= MGPBD_STATUS_CG_MAXITER;
    }
  }
}

// Restart of a CG solve from its current iterate: rz from the partials,
// the status bits in clear_mask dropped; iteration count and tolerance kept.
__global__ void k_cg_restart(CgState* st, const double* __restrict__ p, int blocks,
                             int32_t clear_mask) {
  double rz = sum_partials(p, blocks);
  if (threadIdx.x == 0) {
    st->rz = rz;
    st->status &= ~clear_mask;
    if (!isfinite(rz)) st->status |= MGPBD_STATUS_NAN;
    st->done = (st->iters >= st->maxiter || !isfinite(rz)) ? 1 : 0;
  }
}

__global__ void k_cg_update_p(const CgState* __restrict__ st, const float* __restrict__ z,
                              float* __restrict__ p, int64_t n) {
  if (st->done) return;
  float bt = (float)st->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + bt * p[i];
}

// ---------------------------------------------------------------------------
// Dense float64 Cholesky of the coarsest matrix (one block; n small).
__global__ void k_chol_factor(int32_t n, const int32_t* __restrict__ indptr,
                              const int32_t* __restrict__ indices, const float* __restrict__ data,
                              double* __restrict__ L, int32_t* info) {
  // densify (row-major, lower triangle used)
  for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += blockDim.x) L[e] = 0.0;
  __syncthreads();
  for (int32_t i = threadIdx.x; i < n; i += blockDim.x)
    for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) L[(int64_t)i * n + indices[k]] = (double)data[k];
  __syncthreads();
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  // right-looking column Cholesky
  for (int32_t j = 0; j < n; ++j) {
    __shared__ double djj;
    if (threadIdx.x == 0) {
      double d = L[(int64_t)j * n + j];
      if (!(d > 0.0)) {
        bad = 1;
        d = 1.0;
      }
      djj = sqrt(d);
      L[(int64_t)j * n + j] = djj;
    }
    __syncthreads();
    for (int32_t i = j + 1 + threadIdx.x; i < n; i += blockDim.x) L[(int64_t)i * n + j] /= djj;
    __syncthreads();
    // trailing update of the lower triangle
    int64_t m = n - j - 1;
    for (int64_t e = threadIdx.x; e < m * m; e += blockDim.x) {
      int32_t r = j + 1 + (int32_t)(e / m), c = j + 1 + (int32_t)(e % m);
      if (c <= r) L[(int64_t)r * n + c] -= L[(int64_t)r * n + j] * L[(int64_t)c * n + j];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *info = bad;
}

__global__ void k_chol_solve(const CgState* __restrict__ st, const double* __restrict__ L,
                             int32_t n, const float* __restrict__ b, float* __restrict__ x) {
  if (st && st->done) return;
  extern __shared__ double y[];
  for (int32_t i = threadIdx.x; i < n; i += blockDim.x) y[i] = (double)b[i];
  __syncthreads();
  // forward: L y = b
  for (int32_t j = 0; j < n; ++j) {
    if (threadIdx.x == 0) y[j] /= L[(int64_t)j * n + j];
    __syncthreads();
    double yj = y[j];
    for (int32_t i = j + 1 + threadIdx.x; i < n; i += blockDim.x) y[i] -= L[(int64_t)i * n + j] * yj;
    __syncthreads();
  }
  // backward: L^T x = y
  for (int32_t j = n - 1; j >= 0; --j) {
    if (threadIdx.x == 0) y[j] /= L[(int64_t)j * n + j];
    __syncthreads();
    double yj = y[j];
    for (int32_t i = threadIdx.x; i < j; i += blockDim.x) y[i] -= L[(int64_t)j * n + i] * yj;
    __syncthreads();
  }
  for (int32_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = (float)y[i];
}

}  // namespace

// ===========================================================================
int reduce_blocks(int64_t n) { return grid_for(n, kThreads * 4); }

void launch_rest_shape(const float* x_ref, const int32_t* t_i, const int32_t* ctype, int32_t nt,
                       float mu, float dt, float* dm_inv, float* rest_vol, float* alpha,
                       cudaStream_t s) {
  if (nt <= 0) return;
  k_rest_shape<<<grid_for(nt, kThreads), kThreads, 0, s>>>(
      x_ref, reinterpret_cast<const int4*>(t_i), ctype, nt, mu, dt, dm_inv, rest_vol, alpha);
  MGPBD_CHECK_LAUNCH();
}
void launch_constraints(const float* x, const int32_t* t_i, const int32_t* ctype,
                        const float* dm_inv, const float* rest, int32_t nt, float* C,
                        float* gradC, cudaStream_t s) {
  if (nt <= 0) return;
  k_constraints<<<ceil_div(nt, 128), 128, 0, s>>>(x, reinterpret_cast<const int4*>(t_i), ctype,
                                                  dm_inv, rest, nt, C,
                                                  reinterpret_cast<float4*>(gradC));
  MGPBD_CHECK_LAUNCH();
}
void launch_predict(float* x, float* v, float* x_old, float* x_pred, const float* invm, int32_t nv,
                    float dt, const float* g, float damp, int kinematic, cudaStream_t s) {
  if (nv <= 0) return;
  k_predict<<<grid_for(nv, kThreads), kThreads, 0, s>>>(x, v, x_old, x_pred, invm, nv, dt, g[0], g[1],
                                                        g[2], damp, kinematic);
  MGPBD_CHECK_LAUNCH();
}

void launch_update_vel(const float* x, const float* x_old, float* v, int32_t nv, float dt, float damp,
                       cudaStream_t s) {
  if (nv <= 0) return;
  k_update_vel<<<grid_for(nv, kThreads), kThreads, 0, s>>>(x, x_old, v, nv, dt, damp);
  MGPBD_CHECK_LAUNCH();
}

void launch_rhs(const float* C, const float* alpha, const float* lambda, int32_t nt, float* b,
                double* partials, cudaStream_t s) {
  k_rhs<<<reduce_blocks(nt), kThreads, 0, s>>>(C, alpha, lambda, nt, b, partials);
  MGPBD_CHECK_LAUNCH();
}

void launch_dual_sq(const float* C, const float* alpha, const float* lambda, int32_t nt,
                    double* partials, cudaStream_t s) {
  k_rhs<<<reduce_blocks(nt), kThreads, 0, s>>>(C, alpha, lambda, nt, nullptr, partials);
  MGPBD_CHECK_LAUNCH();
}

void launch_dual_trial(const float* x, const float* dpos, const double* omegas, int n_omega,
                       const int32_t* t_i, const int32_t* ctype, const float* dm_inv,
                       const float* rest, const float* alpha, const float* lambda, int32_t nt,
                       double* partials, cudaStream_t s) {
  require(n_omega >= 1 && n_omega <= kMaxOmega, MGPBD_EINVAL, "n_omega out of range");
  k_dual_trial<<<reduce_blocks(nt), kThreads, 0, s>>>(x, dpos, omegas, n_omega,
                                                      reinterpret_cast<const int4*>(t_i), ctype,
                                                      dm_inv, rest, alpha, lambda, nt, partials);
  MGPBD_CHECK_LAUNCH();
}

void launch_chunk_dual_sq(const float* C, const float* alpha, const float* lambda,
                          const int32_t* chunks, int32_t n_chunks, double* partials,
                          cudaStream_t s) {
  if (n_chunks <= 0) return;
  k_chunk_dual_sq<<<n_chunks, kThreads, 0, s>>>(C, alpha, lambda,
                                                reinterpret_cast<const int2*>(chunks), partials);
  MGPBD_CHECK_LAUNCH();
}

void launch_chunk_trial(const float* x, const float* dpos, const double* omegas, int n_omega,
                        const int32_t* t_i, const int32_t* ctype, const float* dm_inv,
                        const float* rest, const float* alpha, const float* lambda,
                        const int32_t* chunks, int32_t n_chunks, double* partials,
                        cudaStream_t s) {
  require(n_omega >= 1 && n_omega <= kMaxOmega, MGPBD_EINVAL, "n_omega out of range");
  if (n_chunks <= 0) return;
  k_chunk_trial<<<n_chunks, kThreads, 0, s>>>(x, dpos, omegas, n_omega,
                                              reinterpret_cast<const int4*>(t_i), ctype, dm_inv,
                                              rest, alpha, lambda,
                                              reinterpret_cast<const int2*>(chunks), partials);
  MGPBD_CHECK_LAUNCH();
}

void launch_mask_rhs(float* b, const int32_t* cons_body, const int32_t* active, int32_t nt,
                     cudaStream_t s) {
  if (nt <= 0) return;
  k_mask_rhs<<<grid_for(nt, kThreads), kThreads, 0, s>>>(b, cons_body, active, nt);
  MGPBD_CHECK_LAUNCH();
}

void launch_apply_bodies(float* x, const float* dpos, const float* invm, const int32_t* vert_body,
                         const float* omega, int32_t nv, cudaStream_t s) {
  if (nv <= 0) return;
  k_apply_bodies<<<grid_for(nv, kThreads), kThreads, 0, s>>>(x, dpos, invm, vert_body, omega, nv);
  MGPBD_CHECK_LAUNCH();
}

void launch_lambda_update(float* lambda, const float* dlam, int32_t nt, cudaStream_t s) {
  if (nt <= 0) return;
  k_lambda_update<<<grid_for(nt, kThreads), kThreads, 0, s>>>(lambda, dlam, nt);
  MGPBD_CHECK_LAUNCH();
}

void launch_scatter(const int32_t* inc_ptr, const int32_t* inc_ent, const float* invm,
                    const float* dlam, const float* gradC, float* dpos, int32_t nv, cudaStream_t s,
                    const float* dlam_lo) {
  if (nv <= 0) return;
  k_scatter<<<grid_for(nv, kThreads), kThreads, 0, s>>>(inc_ptr, inc_ent, invm, dlam, dlam_lo,
                                                        gradC, dpos, nv);
  MGPBD_CHECK_LAUNCH();
}

void launch_apply(float* x, const float* dpos, const float* invm, int32_t nv, float omega,
                  cudaStream_t s) {
  if (nv <= 0) return;
  k_apply<<<grid_for(nv, kThreads), kThreads, 0, s>>>(x, dpos, invm, nv, omega);
  MGPBD_CHECK_LAUNCH();
}

void launch_fill_A(const int32_t* indptr, const int32_t* indices, const int32_t* t_i,
                   const float* invm, const float* gradC, const float* alpha, int32_t nt,
                   float* data, float* diag_inv, cudaStream_t s) {
  if (nt <= 0) return;
  k_fill_A<<<grid_for((int64_t)nt * 32, kThreads), kThreads, 0, s>>>(
      indptr, indices, reinterpret_cast<const int4*>(t_i), invm,
      reinterpret_cast<const float4*>(gradC), alpha, nt, data, diag_inv);
  MGPBD_CHECK_LAUNCH();
}

void launch_rap_refill(const int32_t* off, const int32_t* idx, const float* fine, int64_t nnz_c,
                       float* coarse, cudaStream_t s) {
  if (nnz_c <= 0) return;
  k_rap_refill<<<grid_for(nnz_c, kThreads), kThreads, 0, s>>>(off, idx, fine, nnz_c, coarse);
  MGPBD_CHECK_LAUNCH();
}

void launch_diag_inv_pos(const int32_t* diag_pos, const float* data, int32_t n, float* diag_inv,
                         cudaStream_t s) {
  if (n <= 0) return;
  k_diag_inv_pos<<<grid_for(n, kThreads), kThreads, 0, s>>>(diag_pos, data, n, diag_inv);
  MGPBD_CHECK_LAUNCH();
}

void launch_diag_inv_scan(const int32_t* indptr, const int32_t* indices, const float* data, int32_t n,
                          float* diag_inv, cudaStream_t s) {
  if (n <= 0) return;
  k_diag_inv_scan<<<grid_for(n, kThreads), kThreads, 0, s>>>(indptr, indices, data, n, diag_inv);
  MGPBD_CHECK_LAUNCH();
}

void launch_spmv(const CsrView& a, const float* x, float* y, cudaStream_t s) {
  rows_dispatch<kSpmv>(a, x, nullptr, y, 0.0f, nullptr, nullptr, s);
}
void launch_spmv_dot(const CsrView& a, const float* x, float* y, double* partials, cudaStream_t s) {
  rows_dispatch<kSpmvDot>(a, x, nullptr, y, 0.0f, partials, nullptr, s);
}
void launch_jacobi(const CsrView& a, const float* b, const float* x, float* x_new, float w,
                   cudaStream_t s) {
  if (x) rows_dispatch<kJacobi>(a, x, b, x_new, w, nullptr, nullptr, s);
  else rows_dispatch<kJacobiZero>(a, nullptr, b, x_new, w, nullptr, nullptr, s);
}
void launch_residual(const CsrView& a, const float* b, const float* x, float* r, cudaStream_t s) {
  rows_dispatch<kResidual>(a, x, b, r, 0.0f, nullptr, nullptr, s);
}
void launch_restrict(const int32_t* mem_ptr, const int32_t* mem_rows, const float* r, int32_t nc,
                     float* bc, cudaStream_t s) {
  launch_restrict_g(nullptr, mem_ptr, mem_rows, r, nc, bc, s);
}
void launch_prolong_add(const int32_t* agg, const float* xc, int32_t n, float* x, cudaStream_t s) {
  launch_prolong_add_g(nullptr, agg, xc, n, x, s);
}

void launch_jacobi_g(const CgState* st, const CsrView& a, const float* b, const float* x, float* x_new,
                     float w, cudaStream_t s) {
  if (x) rows_dispatch<kJacobi>(a, x, b, x_new, w, nullptr, st, s);
  else rows_dispatch<kJacobiZero>(a, nullptr, b, x_new, w, nullptr, st, s);
}
void launch_jacobi_gw(const CgState* st, const CsrView& a, const float* b, const float* x,
                      float* x_new, float w, const float* w_dev, cudaStream_t s) {
  if (x) rows_dispatch<kJacobi>(a, x, b, x_new, w, nullptr, st, s, w_dev);
  else rows_dispatch<kJacobiZero>(a, nullptr, b, x_new, w, nullptr, st, s, w_dev);
}
void launch_residual_g(const CgState* st, const CsrView& a, const float* b, const float* x, float* r,
                       cudaStream_t s) {
  rows_dispatch<kResidual>(a, x, b, r, 0.0f, nullptr, st, s);
}
void launch_restrict_g(const CgState* st, const int32_t* mem_ptr, const int32_t* mem_rows,
                       const float* r, int32_t nc, float* bc, cudaStream_t s) {
  if (nc <= 0) return;
  k_restrict<<<grid_for(nc, kThreads), kThreads, 0, s>>>(mem_ptr, mem_rows, r, nc, bc, st);
  MGPBD_CHECK_LAUNCH();
}
void launch_prolong_add_g(const CgState* st, const int32_t* agg, const float* xc, int32_t n, float* x,
                          cudaStream_t s) {
  if (n <= 0) return;
  k_prolong_add<<<grid_for(n, kThreads), kThreads, 0, s>>>(agg, xc, n, x, st);
  MGPBD_CHECK_LAUNCH();
}
void launch_spmv_dot_g(const CgState* st, const CsrView& a, const float* x, float* y, double* partials,
                       cudaStream_t s) {
  rows_dispatch<kSpmvDot>(a, x, nullptr, y, 0.0f, partials, st, s);
}
void launch_dot_partials_g(const CgState* st, const float* a, const float* b, int64_t n,
                           double* partials, cudaStream_t s) {
  k_dot<<<reduce_blocks(n), kThreads, 0, s>>>(a, b, n, partials, st);
  MGPBD_CHECK_LAUNCH();
}

void launch_dot_partials(const float* a, const float* b, int64_t n, double* partials, cudaStream_t s) {
  launch_dot_partials_g(nullptr, a, b, n, partials, s);
}
void launch_axpy(float alpha, const float* x, float* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  k_axpy<<<grid_for(n, kThreads), kThreads, 0, s>>>(alpha, x, y, n);
  MGPBD_CHECK_LAUNCH();
}
void launch_scale(float alpha, float* x, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  k_scale<<<grid_for(n, kThreads), kThreads, 0, s>>>(alpha, x, n);
  MGPBD_CHECK_LAUNCH();
}
void launch_xpay(float alpha, const float* x, float* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  k_xpay<<<grid_for(n, kThreads), kThreads, 0, s>>>(alpha, x, y, n);
  MGPBD_CHECK_LAUNCH();
}
void launch_finalize(const double* partials, int blocks, int count, double* out, cudaStream_t s) {
  k_finalize<<<1, kThreads, 0, s>>>(partials, blocks, count, out);
  MGPBD_CHECK_LAUNCH();
}

void launch_cg_init(CgState* st, const double* partials_rz, int blocks, double tol_abs, double tol_rel,
                    int maxiter, cudaStream_t s) {
  k_cg_init<<<1, kThreads, 0, s>>>(st, partials_rz, blocks, tol_abs, tol_rel, maxiter);
  MGPBD_CHECK_LAUNCH();
}
void launch_cg_alpha(CgState* st, const double* p, int blocks, cudaStream_t s) {
  k_cg_alpha<<<1, kThreads, 0, s>>>(st, p, blocks);
  MGPBD_CHECK_LAUNCH();
}
void launch_cg_update_xr(const CgState* st, const float* p, const float* ap, float* x, float* r,
                         int64_t n, double* partials, cudaStream_t s) {
  k_cg_update_xr<<<reduce_blocks(n), kThreads, 0, s>>>(st, p, ap, x, r, n, partials);
  MGPBD_CHECK_LAUNCH();
}
void launch_cg_check(CgState* st, const double* p, int blocks, cudaStream_t s) {
  k_cg_check<<<1, kThreads, 0, s>>>(st, p, blocks);
  MGPBD_CHECK_LAUNCH();
}
void launch_cg_beta(CgState* st, const double* p, int blocks, cudaStream_t s) {
  k_cg_beta<<<1, kThreads, 0, s>>>(st, p, blocks);
  MGPBD_CHECK_LAUNCH();
}
void launch_cg_restart(CgState* st, const double* p, int blocks, int32_t clear_mask,
                       cudaStream_t s) {
  k_cg_restart<<<1, kThreads, 0, s>>>(st, p, blocks, clear_mask);
  MGPBD_CHECK_LAUNCH();
}
void launch_cg_update_p(const CgState* st, const float* z, float* p, int64_t n, cudaStream_t s) {
  k_cg_update_p<<<grid_for(n, kThreads), kThreads, 0, s>>>(st, z, p, n);
  MGPBD_CHECK_LAUNCH();
}

void launch_dense_chol_factor(const CsrView& a, double* work, int32_t n, int32_t* info, cudaStream_t s) {
  k_chol_factor<<<1, 1024, 0, s>>>(n, a.indptr, a.indices, a.data, work, info);
  MGPBD_CHECK_LAUNCH();
}
void launch_dense_chol_solve(const CgState* st, const double* L, int32_t n, const float* b, float* x,
                             cudaStream_t s) {
  k_chol_solve<<<1, 256, sizeof(double) * n, s>>>(st, L, n, b, x);
  MGPBD_CHECK_LAUNCH();
}

int row_shape_code(int idx) {
  require(idx >= 0 && idx < kNumRowShapes, MGPBD_EINVAL, "row shape index out of range");
  return 100 * kRowShapeG[idx] + kRowShapeU[idx];
}

int row_shape_index(int code) {
  for (int i = 0; i < kNumRowShapes; ++i)
    if (100 * kRowShapeG[i] + kRowShapeU[i] == code) return i;
  throw Error(MGPBD_EINVAL, "unknown row-kernel shape code (G * 100 + U)");
}

int tune_row_shape(const CsrView& a, const float* x, const float* b, float* y, int reps,
                   cudaStream_t s, float* best_us) {
  require(a.padded, MGPBD_EINVAL, "tune_row_shape needs a padded (library) CSR matrix");
  require(reps >= 1, MGPBD_EINVAL, "tune_row_shape: reps must be positive");
  cudaEvent_t e0, e1;
  MGPBD_CUDA(cudaEventCreate(&e0));
  MGPBD_CUDA(cudaEventCreate(&e1));
  int best = 0;
  float best_ms = 0.f;
  try {
    for (int i = 0; i < kNumRowShapes; ++i) {
      launch_vec_shape<kJacobi>(i, a, x, b, y, 0.5f, nullptr, nullptr, s, nullptr);
      MGPBD_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < reps; ++r)
        launch_vec_shape<kJacobi>(i, a, x, b, y, 0.5f, nullptr, nullptr, s, nullptr);
      MGPBD_CUDA(cudaEventRecord(e1, s));
      MGPBD_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      MGPBD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (i == 0 || ms < best_ms) {
        best_ms = ms;
        best = i;
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_us) *best_us = 1e3f * best_ms / reps;
  return best;
}

}  // namespace mgpbd
