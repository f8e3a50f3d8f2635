// Learned coarse correction: forward, backward and Adam kernels of the
// message-passing network declared in mpnn.cuh.
//
// Forward per application (5 launches): partials of |S r|^2, their sum,
// layer 1 (scalar message passing, warp per row), then two fused layer
// kernels, each one CTA per 64 aggregates:
//   1. copy the 64 rows of H (bf16) and aggregate Ah H for them (a quarter
//      warp per neighbour, 16-byte loads of the neighbour's 64 features,
//      float32 sums) into a shared 64 x 128 bf16 tile X = [H, Ah H];
//   2. X (64 x 128) . W (128 x 64) on the tensor cores (mma.sync m16n8k16,
//      bf16 operands, float32 accumulation), W^T staged in shared memory;
//   3. bias + relu, written back as bf16 (or, in the last layer, reduced
//      against wo to the output and scaled to the correction).
// Backward (training only) is float32 on the CUDA cores: weight gradients
// are per-block partial sums added in a fixed order (deterministic).
#include "mpnn.cuh"

#include <cmath>
#include <vector>

#include "kernels.cuh"

namespace mgpbd {

namespace {

constexpr int kT = 256;           // threads of the row-parallel kernels
constexpr int kLayerRows = 64;    // aggregates per layer CTA
constexpr int kLayerThreads = 128;
constexpr int kXS = 136;          // padded bf16 row stride of the shared tiles
constexpr int kWgradBlocks = 304; // 2 x 152 SMs
constexpr int kBigPart = 2 * kNetF * kNetF + kNetF;  // W (128 x 64) + b
// weights stay below kNetWeightBound / sum_j |Ah_ij| (< 2 / sum: no mode is
// over-corrected, Gershgorin)
constexpr float kNetWeightBound = 1.9f;

__device__ __forceinline__ float scale_of(const float* __restrict__ dinv, int i) {
  float d = dinv[i];
  return d > 0.f ? sqrtf(d) : 0.f;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// float64 block sum in a fixed pattern; valid in thread 0
__device__ __forceinline__ double block_sum_d(double v) {
  __shared__ double sh[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum_d(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum_d(v);
  __syncthreads();
  return v;
}

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a (low half)
  return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---- forward ---------------------------------------------------------------

// partials of sum_i (s_i r_i)^2
__global__ void k_net_sumsq(int32_t n, const float* __restrict__ r,
                            const float* __restrict__ dinv, double* __restrict__ part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float v = scale_of(dinv, (int)i) * r[i];
    acc += (double)v * (double)v;
  }
  acc = block_sum_d(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void k_net_sum(const double* __restrict__ part, int blocks, double* __restrict__ out,
                          int accumulate) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < blocks; i += blockDim.x) acc += part[i];
  acc = block_sum_d(acc);
  if (threadIdx.x == 0) out[0] = accumulate ? out[0] + acc : acc;
}

__device__ __forceinline__ float inv_sigma(const double* sumsq, int32_t n) {
  double ss = *sumsq;
  return ss > 0.0 ? (float)(1.0 / sqrt(ss / (double)n)) : 0.f;
}

// layer 1: warp per aggregate; H1 = relu(u w1s + (Ah u) w1n + b1)
__global__ void __launch_bounds__(kT) k_net_l1(NetGraph g, const float* __restrict__ r,
                                               const double* __restrict__ sumsq,
                                               const float* __restrict__ P,
                                               __nv_bfloat16* __restrict__ H1,
                                               float* __restrict__ ah,
                                               float* __restrict__ cap_out,
                                               float* __restrict__ u_out,
                                               float* __restrict__ a1_out) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * (kT / 32) + (threadIdx.x >> 5);
  if (row >= g.n) return;
  const float inv = inv_sigma(sumsq, g.n);
  const float si = scale_of(g.diag_inv, row);
  const float ui = si * r[row] * inv;
  float acc = 0.f;  // sum_j Ah_ij u_j; Ah_ij = s_i A_ij s_j kept for the layers
  float rabs = 0.f;  // sum_j |Ah_ij|
  for (int k = g.indptr[row] + lane; k < g.indptr[row + 1]; k += 32) {
    const int j = g.indices[k];
    const float sj = scale_of(g.diag_inv, j);
    const float a = g.data[k] * si * sj;
    ah[k] = a;
    acc += a * (sj * r[j] * inv);
    rabs += fabsf(a);
  }
  const float a1 = warp_sum_f(acc);
  if (cap_out) {
    rabs = warp_sum_f(rabs);
    if (lane == 0) cap_out[row] = rabs > 0.f ? kNetWeightBound / rabs : 0.f;
  }
  const float2 ws = reinterpret_cast<const float2*>(P + kNetOffW1s)[lane];
  const float2 wn = reinterpret_cast<const float2*>(P + kNetOffW1n)[lane];
  const float2 b = reinterpret_cast<const float2*>(P + kNetOffB1)[lane];
  float z0 = fmaxf(ui * ws.x + a1 * wn.x + b.x, 0.f);
  float z1 = fmaxf(ui * ws.y + a1 * wn.y + b.y, 0.f);
  reinterpret_cast<uint32_t*>(H1 + (int64_t)row * kNetF)[lane] = pack_bf2(z0, z1);
  if (u_out && lane == 0) {
    u_out[row] = ui;
    a1_out[row] = a1;
  }
}

// layers 2 and 3 (see the file comment).  Not last: Hn = relu(X W + b) as
// bf16.  Last: y = relu(X W + b) . wo + bo, e = sigma s y (and, for
// training, y and the float32 activations h3).
template <bool kLast>
__global__ void __launch_bounds__(kLayerThreads) k_net_layer(
    NetGraph g, const float* __restrict__ ah, const __nv_bfloat16* __restrict__ H,
    const __nv_bfloat16* __restrict__ Wt, const float* __restrict__ P, int bias_off,
    __nv_bfloat16* __restrict__ Hn,
    __nv_bfloat16* __restrict__ Gout, const double* __restrict__ sumsq, float* __restrict__ y_out,
    float* __restrict__ e_out, float* __restrict__ h3_out) {
  __shared__ __align__(16) __nv_bfloat16 Xs[kLayerRows * kXS];
  __shared__ __align__(16) __nv_bfloat16 Ws[kNetF * kXS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int row0 = blockIdx.x * kLayerRows;

  for (int c = tid; c < kNetF * 16; c += kLayerThreads) {
    int o = c >> 4, k8 = c & 15;
    *reinterpret_cast<uint4*>(Ws + o * kXS + k8 * 8) =
        *reinterpret_cast<const uint4*>(Wt + o * 2 * kNetF + k8 * 8);
  }
  for (int c = tid; c < kLayerRows * 8; c += kLayerThreads) {
    int r = c >> 3, k8 = c & 7;
    int row = row0 + r;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (row < g.n) v = *reinterpret_cast<const uint4*>(H + (int64_t)row * kNetF + k8 * 8);
    *reinterpret_cast<uint4*>(Xs + r * kXS + k8 * 8) = v;
  }

  // G = Ah H for this CTA's rows: warp w takes rows 16w..16w+15.  The warp
  // loads up to 32 (column, Ah) pairs of a row at once; each quarter warp
  // then gathers four neighbours' 64 features (16 bytes a lane) before
  // using any, so 16 neighbour rows are in flight per warp.
  const int grp = lane >> 3, sub = lane & 7;
  for (int rr = 0; rr < 16; ++rr) {
    const int r = warp * 16 + rr;
    const int row = row0 + r;
    float acc[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) acc[t] = 0.f;
    if (row < g.n) {  // uniform across the warp
      const int k0 = g.indptr[row], k1 = g.indptr[row + 1];
      for (int base = k0; base < k1; base += 32) {
        const int cnt = min(32, k1 - base);
        int jl = 0;
        float al = 0.f;
        if (lane < cnt) {
          jl = g.indices[base + lane];
          al = ah[base + lane];
        }
        for (int t0 = 0; t0 < cnt; t0 += 16) {
          uint4 hv[4];
          float a[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int idx = t0 + grp + 4 * u;
            const int jj = __shfl_sync(0xffffffffu, jl, idx & 31);
            const float aa = __shfl_sync(0xffffffffu, al, idx & 31);
            if (idx < cnt) {
              hv[u] = *reinterpret_cast<const uint4*>(H + (int64_t)jj * kNetF + sub * 8);
              a[u] = aa;
            } else {
              hv[u] = make_uint4(0u, 0u, 0u, 0u);
              a[u] = 0.f;
            }
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            acc[0] += a[u] * bf_lo(hv[u].x);
            acc[1] += a[u] * bf_hi(hv[u].x);
            acc[2] += a[u] * bf_lo(hv[u].y);
            acc[3] += a[u] * bf_hi(hv[u].y);
            acc[4] += a[u] * bf_lo(hv[u].z);
            acc[5] += a[u] * bf_hi(hv[u].z);
            acc[6] += a[u] * bf_lo(hv[u].w);
            acc[7] += a[u] * bf_hi(hv[u].w);
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      acc[t] += __shfl_xor_sync(0xffffffffu, acc[t], 8);
      acc[t] += __shfl_xor_sync(0xffffffffu, acc[t], 16);
    }
    if (grp == 0) {
      uint4 o;
      o.x = pack_bf2(acc[0], acc[1]);
      o.y = pack_bf2(acc[2], acc[3]);
      o.z = pack_bf2(acc[4], acc[5]);
      o.w = pack_bf2(acc[6], acc[7]);
      *reinterpret_cast<uint4*>(Xs + r * kXS + kNetF + sub * 8) = o;
      if (Gout && row < g.n)
        *reinterpret_cast<uint4*>(Gout + (int64_t)row * kNetF + sub * 8) = o;
    }
  }
  __syncthreads();

  // X (rows 16w..16w+15) . W on the tensor cores
  float acc[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
  const int gq = lane >> 2, tq = lane & 3;
  const __nv_bfloat16* xa = Xs + (warp * 16 + gq) * kXS + 2 * tq;
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const uint32_t a0 = *reinterpret_cast<const uint32_t*>(xa + kk * 16);
    const uint32_t a1 = *reinterpret_cast<const uint32_t*>(xa + 8 * kXS + kk * 16);
    const uint32_t a2 = *reinterpret_cast<const uint32_t*>(xa + kk * 16 + 8);
    const uint32_t a3 = *reinterpret_cast<const uint32_t*>(xa + 8 * kXS + kk * 16 + 8);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const __nv_bfloat16* wb = Ws + (nt * 8 + gq) * kXS + kk * 16 + 2 * tq;
      mma_bf16(acc[nt], a0, a1, a2, a3, *reinterpret_cast<const uint32_t*>(wb),
               *reinterpret_cast<const uint32_t*>(wb + 8));
    }
  }

  const int rA = warp * 16 + gq, rB = rA + 8;
  const int rowA = row0 + rA, rowB = row0 + rB;
  if (!kLast) {
    __syncwarp();  // this warp's MMAs have read its rows of Xs
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int c = nt * 8 + 2 * tq;
      const float b0 = P[bias_off + c], b1 = P[bias_off + c + 1];
      *reinterpret_cast<uint32_t*>(Xs + rA * kXS + c) =
          pack_bf2(fmaxf(acc[nt][0] + b0, 0.f), fmaxf(acc[nt][1] + b1, 0.f));
      *reinterpret_cast<uint32_t*>(Xs + rB * kXS + c) =
          pack_bf2(fmaxf(acc[nt][2] + b0, 0.f), fmaxf(acc[nt][3] + b1, 0.f));
    }
    __syncwarp();
    for (int c = lane; c < 16 * 8; c += 32) {
      const int r = warp * 16 + (c >> 3), k8 = c & 7;
      const int row = row0 + r;
      if (row < g.n)
        *reinterpret_cast<uint4*>(Hn + (int64_t)row * kNetF + k8 * 8) =
            *reinterpret_cast<const uint4*>(Xs + r * kXS + k8 * 8);
    }
  } else {
    float ya = 0.f, yb = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int c = nt * 8 + 2 * tq;
      const float b0 = P[bias_off + c], b1 = P[bias_off + c + 1];
      const float w0 = P[kNetOffWo + c], w1 = P[kNetOffWo + c + 1];
      const float ha0 = fmaxf(acc[nt][0] + b0, 0.f), ha1 = fmaxf(acc[nt][1] + b1, 0.f);
      const float hb0 = fmaxf(acc[nt][2] + b0, 0.f), hb1 = fmaxf(acc[nt][3] + b1, 0.f);
      ya += ha0 * w0 + ha1 * w1;
      yb += hb0 * w0 + hb1 * w1;
      if (h3_out) {
        if (rowA < g.n)
          *reinterpret_cast<float2*>(h3_out + (int64_t)rowA * kNetF + c) = make_float2(ha0, ha1);
        if (rowB < g.n)
          *reinterpret_cast<float2*>(h3_out + (int64_t)rowB * kNetF + c) = make_float2(hb0, hb1);
      }
    }
    ya += __shfl_xor_sync(0xffffffffu, ya, 1);
    ya += __shfl_xor_sync(0xffffffffu, ya, 2);
    yb += __shfl_xor_sync(0xffffffffu, yb, 1);
    yb += __shfl_xor_sync(0xffffffffu, yb, 2);
    if (tq == 0) {
      const float bo = P[kNetOffBo];
      const double ss = *sumsq;
      const float sigma = ss > 0.0 ? (float)sqrt(ss / (double)g.n) : 0.f;
      ya += bo;
      yb += bo;
      if (rowA < g.n) {
        if (y_out) y_out[rowA] = ya;
        e_out[rowA] = sigma * scale_of(g.diag_inv, rowA) * ya;
      }
      if (rowB < g.n) {
        if (y_out) y_out[rowB] = yb;
        e_out[rowB] = sigma * scale_of(g.diag_inv, rowB) * yb;
      }
    }
  }
}

// ---- backward (training) ---------------------------------------------------

// Output layer: gy = (Ah y - u) * scale, gZ3 = gy wo^T masked by h3 > 0,
// block partials of the loss (1/2 y Ah y - y u) * scale.  Warp per row,
// rows strided over a fixed grid so the partials are deterministic.
__global__ void __launch_bounds__(kT) k_net_out_bwd(NetGraph g, const float* __restrict__ ah,
                                                    const float* __restrict__ y,
                                                    const float* __restrict__ u,
                                                    const float* __restrict__ h3,
                                                    const float* __restrict__ P, float scale,
                                                    float* __restrict__ gy_out,
                                                    float* __restrict__ gz,
                                                    double* __restrict__ loss_part) {
  const int lane = threadIdx.x & 31;
  const int wpb = kT / 32;
  double lacc = 0.0;
  const float2 wo = reinterpret_cast<const float2*>(P + kNetOffWo)[lane];
  for (int row = blockIdx.x * wpb + (threadIdx.x >> 5); row < g.n; row += gridDim.x * wpb) {
    float acc = 0.f;
    for (int k = g.indptr[row] + lane; k < g.indptr[row + 1]; k += 32)
      acc += ah[k] * y[g.indices[k]];
    const float ay = warp_sum_f(acc);
    const float yi = y[row], ui = u[row];
    const float gy = (ay - ui) * scale;
    if (lane == 0) {
      gy_out[row] = gy;
      lacc += (0.5 * (double)yi * (double)ay - (double)yi * (double)ui) * (double)scale;
    }
    const float2 h = reinterpret_cast<const float2*>(h3 + (int64_t)row * kNetF)[lane];
    reinterpret_cast<float2*>(gz + (int64_t)row * kNetF)[lane] =
        make_float2(h.x > 0.f ? gy * wo.x : 0.f, h.y > 0.f ? gy * wo.y : 0.f);
  }
  lacc = block_sum_d(lacc);
  if (threadIdx.x == 0) loss_part[blockIdx.x] = lacc;
}

// Weights form, per sample: u = S r / sigma_r, v = w * u (w the squashed
// weights, dw = dw/dy), gy += (Ah v - u) * u * dw * scale, loss partials of
// (1/2 v^T Ah v - v^T u) * scale.  Warp per row over a fixed grid.
__global__ void __launch_bounds__(kT) k_net_wloss(NetGraph g, const float* __restrict__ ah,
                                                  const float* __restrict__ w,
                                                  const float* __restrict__ dw,
                                                  const float* __restrict__ r,
                                                  const double* __restrict__ sumsq, float scale,
                                                  float* __restrict__ gy,
                                                  double* __restrict__ loss_part) {
  const int lane = threadIdx.x & 31;
  const int wpb = kT / 32;
  const float inv = inv_sigma(sumsq, g.n);
  double lacc = 0.0;
  for (int row = blockIdx.x * wpb + (threadIdx.x >> 5); row < g.n; row += gridDim.x * wpb) {
    float acc = 0.f;
    for (int k = g.indptr[row] + lane; k < g.indptr[row + 1]; k += 32) {
      const int j = g.indices[k];
      acc += ah[k] * (w[j] * (scale_of(g.diag_inv, j) * r[j] * inv));
    }
    const float av = warp_sum_f(acc);
    if (lane == 0) {
      const float ui = scale_of(g.diag_inv, row) * r[row] * inv;
      const float vi = w[row] * ui;
      gy[row] += (av - ui) * ui * dw[row] * scale;
      lacc += (0.5 * (double)vi * (double)av - (double)vi * (double)ui) * (double)scale;
    }
  }
  lacc = block_sum_d(lacc);
  if (threadIdx.x == 0) loss_part[blockIdx.x] = lacc;
}

// gz3 = gy wo^T masked by h3 > 0 (the head's backward)
__global__ void k_net_head_bwd(int32_t n, const float* __restrict__ gy,
                               const float* __restrict__ h3, const float* __restrict__ P,
                               float* __restrict__ gz) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)n * kNetF) return;
  const int f = (int)(i & (kNetF - 1));
  gz[i] = h3[i] > 0.f ? gy[i >> 6] * P[kNetOffWo + f] : 0.f;
}

// feature field r_i = sqrt(A_ii) (u = 1 after the scaling)
__global__ void k_net_feat(int32_t n, const float* __restrict__ dinv, float* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float s = scale_of(dinv, i);
  f[i] = s > 0.f ? 1.f / s : 0.f;
}

// w = cap * sigmoid(y) (and dw = dw/dy when dw != nullptr)
__global__ void k_net_squash(int32_t n, const float* __restrict__ y, const float* __restrict__ cap,
                             float* __restrict__ w, float* __restrict__ dw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float sg = 1.f / (1.f + expf(-y[i]));
  w[i] = cap[i] * sg;
  if (dw) dw[i] = cap[i] * sg * (1.f - sg);
}

// e = max(w, 0) * dinv * r (the per-V-cycle coarse correction)
__global__ void k_net_apply(int32_t n, const float* __restrict__ w, const float* __restrict__ dinv,
                            const float* __restrict__ r, float* __restrict__ e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  e[i] = fmaxf(w[i], 0.f) * dinv[i] * r[i];
}

// rows [b * chunk, min(n, (b + 1) * chunk)) of block b
__device__ __forceinline__ void block_rows(int32_t n, int& lo, int& hi) {
  int chunk = (n + gridDim.x - 1) / gridDim.x;
  lo = blockIdx.x * chunk;
  hi = min(n, lo + chunk);
}

// partials of [wo | bo]: sum_i h3[i][f] gy_i and sum_i gy_i (65 per block)
__global__ void __launch_bounds__(kT) k_net_wgrad_out(int32_t n, const float* __restrict__ h3,
                                                      const float* __restrict__ gy,
                                                      float* __restrict__ part) {
  __shared__ float sh[4][kNetF + 1];
  const int f = threadIdx.x & 63, rg = threadIdx.x >> 6;
  int lo, hi;
  block_rows(n, lo, hi);
  float acc = 0.f, accb = 0.f;
  for (int i = lo + rg; i < hi; i += 4) {
    const float gi = gy[i];
    acc += h3[(int64_t)i * kNetF + f] * gi;
    accb += gi;
  }
  sh[rg][f] = acc;
  if (f == 0) sh[rg][kNetF] = accb;
  __syncthreads();
  if (threadIdx.x <= kNetF) {
    const int c = threadIdx.x;
    part[(int64_t)blockIdx.x * (kNetF + 1) + c] = (sh[0][c] + sh[1][c]) + (sh[2][c] + sh[3][c]);
  }
}

// partials of [w1s | w1n | b1]: sums of u_i gz, a1_i gz, gz (192 per block)
__global__ void __launch_bounds__(kT) k_net_wgrad_l1(int32_t n, const float* __restrict__ u,
                                                     const float* __restrict__ a1,
                                                     const float* __restrict__ gz,
                                                     float* __restrict__ part) {
  __shared__ float sh[4][3 * kNetF];
  const int f = threadIdx.x & 63, rg = threadIdx.x >> 6;
  int lo, hi;
  block_rows(n, lo, hi);
  float as = 0.f, an = 0.f, ab = 0.f;
  for (int i = lo + rg; i < hi; i += 4) {
    const float z = gz[(int64_t)i * kNetF + f];
    as += u[i] * z;
    an += a1[i] * z;
    ab += z;
  }
  sh[rg][f] = as;
  sh[rg][kNetF + f] = an;
  sh[rg][2 * kNetF + f] = ab;
  __syncthreads();
  for (int c = threadIdx.x; c < 3 * kNetF; c += kT)
    part[(int64_t)blockIdx.x * 3 * kNetF + c] = (sh[0][c] + sh[1][c]) + (sh[2][c] + sh[3][c]);
}

// partials of [W | b] for X = [H, G] (bf16, n x 128) and gz (n x 64):
// W[k][f] = sum_i X[i][k] gz[i][f], b[f] = sum_i gz[i][f].  Thread t owns
// k = t / 2 and the features f = 2 j + (t & 1).
__global__ void __launch_bounds__(kT) k_net_wgrad_big(int32_t n,
                                                      const __nv_bfloat16* __restrict__ H,
                                                      const __nv_bfloat16* __restrict__ G,
                                                      const float* __restrict__ gz,
                                                      float* __restrict__ part) {
  constexpr int kTile = 32;
  __shared__ float xs[kTile][2 * kNetF];
  __shared__ float zs[kTile][kNetF];
  const int t = threadIdx.x, k = t >> 1, par = t & 1;
  int lo, hi;
  block_rows(n, lo, hi);
  float acc[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) acc[j] = 0.f;
  float accb = 0.f;
  for (int base = lo; base < hi; base += kTile) {
    const int rows = min(kTile, hi - base);
    __syncthreads();
    for (int c = t; c < kTile * 2 * kNetF; c += kT) {
      const int r = c >> 7, kk = c & 127;
      float v = 0.f;
      if (r < rows) {
        const int64_t i = base + r;
        v = kk < kNetF ? __bfloat162float(H[i * kNetF + kk]) : __bfloat162float(G[i * kNetF + kk - kNetF]);
      }
      xs[r][kk] = v;
    }
    for (int c = t; c < kTile * kNetF; c += kT) {
      const int r = c >> 6, ff = c & 63;
      zs[r][ff] = r < rows ? gz[(int64_t)(base + r) * kNetF + ff] : 0.f;
    }
    __syncthreads();
    for (int r = 0; r < rows; ++r) {
      const float x = xs[r][k];
#pragma unroll
      for (int j = 0; j < 32; ++j) acc[j] += x * zs[r][2 * j + par];
      if (t < kNetF) accb += zs[r][t];
    }
  }
  float* out = part + (int64_t)blockIdx.x * kBigPart;
#pragma unroll
  for (int j = 0; j < 32; ++j) out[k * kNetF + 2 * j + par] = acc[j];
  if (t < kNetF) out[2 * kNetF * kNetF + t] = accb;
}

// dst[c] += sum_b part[b * count + c], blocks in ascending order
__global__ void k_net_wsum(const float* __restrict__ part, int blocks, int count,
                           float* __restrict__ dst) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= count) return;
  float acc = 0.f;
  for (int b = 0; b < blocks; ++b) acc += part[(int64_t)b * count + c];
  dst[c] += acc;
}

// gX = gz W^T (n x 128): gself = columns 0..63, q = columns 64..127.
// Thread t of the 128 owns input feature k = t; rows in tiles of 32.
__global__ void __launch_bounds__(2 * kNetF) k_net_xgrad(int32_t n, const float* __restrict__ gz,
                                                         const __nv_bfloat16* __restrict__ Wt,
                                                         float* __restrict__ gself,
                                                         float* __restrict__ q) {
  constexpr int kTile = 32;
  __shared__ float wf[kNetF][2 * kNetF];
  __shared__ float zs[kTile][kNetF];
  const int t = threadIdx.x;
  for (int c = t; c < kNetF * 2 * kNetF; c += blockDim.x)
    wf[c >> 7][c & 127] = __bfloat162float(Wt[c]);
  const int base = blockIdx.x * kTile;
  for (int c = t; c < kTile * kNetF; c += blockDim.x) {
    const int r = c >> 6, f = c & 63;
    zs[r][f] = base + r < n ? gz[(int64_t)(base + r) * kNetF + f] : 0.f;
  }
  __syncthreads();
  for (int r = 0; r < kTile && base + r < n; ++r) {
    float acc = 0.f;
#pragma unroll 16
    for (int o = 0; o < kNetF; ++o) acc += zs[r][o] * wf[o][t];
    const int64_t i = base + r;
    if (t < kNetF)
      gself[i * kNetF + t] = acc;
    else
      q[i * kNetF + t - kNetF] = acc;
  }
}

// gz_prev = (gself + Ah q) masked by h_prev > 0; warp per row, 2 features a lane
__global__ void __launch_bounds__(kT) k_net_hgrad(NetGraph g, const float* __restrict__ ah,
                                                  const float* __restrict__ gself,
                                                  const float* __restrict__ q,
                                                  const __nv_bfloat16* __restrict__ hprev,
                                                  float* __restrict__ gz) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * (kT / 32) + (threadIdx.x >> 5);
  if (row >= g.n) return;
  float a0 = 0.f, a1 = 0.f;
  for (int k = g.indptr[row]; k < g.indptr[row + 1]; ++k) {
    const float a = ah[k];
    const float2 v = reinterpret_cast<const float2*>(q + (int64_t)g.indices[k] * kNetF)[lane];
    a0 += a * v.x;
    a1 += a * v.y;
  }
  const float2 s = reinterpret_cast<const float2*>(gself + (int64_t)row * kNetF)[lane];
  const uint32_t h = reinterpret_cast<const uint32_t*>(hprev + (int64_t)row * kNetF)[lane];
  reinterpret_cast<float2*>(gz + (int64_t)row * kNetF)[lane] =
      make_float2(bf_lo(h) > 0.f ? s.x + a0 : 0.f, bf_hi(h) > 0.f ? s.y + a1 : 0.f);
}

__global__ void k_net_adam(float* __restrict__ p, const float* __restrict__ g,
                           float* __restrict__ m, float* __restrict__ v, int count, float lr,
                           float b1, float b2, float eps, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// Wt[layer][o][k] = bf16(W_layer[k][o]) for layers 2 and 3
__global__ void k_net_pack(const float* __restrict__ p, __nv_bfloat16* __restrict__ wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int kPer = 2 * kNetF * kNetF;
  if (i >= 2 * kPer) return;
  const int layer = i / kPer, rem = i % kPer, o = rem / (2 * kNetF), k = rem % (2 * kNetF);
  const float* W = p + (layer == 0 ? kNetOffW2 : kNetOffW3);
  wt[i] = __float2bfloat16_rn(W[k * kNetF + o]);
}

// splitmix64 (Steele, Lea & Flood 2014) for the seeded initial weights
uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

}  // namespace

// ---- CoarseNet -------------------------------------------------------------

CoarseNet::CoarseNet(uint64_t seed) {
  std::vector<float> h(kNetParams, 0.f);
  uint64_t st = seed;
  auto uni = [&](float bound) {
    double x = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
    return (float)((2.0 * x - 1.0) * bound);
  };
  const float b1 = std::sqrt(6.f / (2 + kNetF)), b2 = std::sqrt(6.f / (3 * kNetF)),
              bo = std::sqrt(6.f / (1 + kNetF));
  for (int i = 0; i < kNetF; ++i) h[kNetOffW1s + i] = uni(b1);
  for (int i = 0; i < kNetF; ++i) h[kNetOffW1n + i] = uni(b1);
  for (int i = 0; i < 2 * kNetF * kNetF; ++i) h[kNetOffW2 + i] = uni(b2);
  for (int i = 0; i < 2 * kNetF * kNetF; ++i) h[kNetOffW3 + i] = uni(b2);
  for (int i = 0; i < kNetF; ++i) h[kNetOffWo + i] = uni(bo);
  p_.alloc(kNetParams);
  g_.alloc(kNetParams);
  m_.alloc(kNetParams);
  v_.alloc(kNetParams);
  wt_.alloc(4 * kNetF * kNetF);
  MGPBD_CUDA(cudaMemcpy(p_.p, h.data(), sizeof(float) * kNetParams, cudaMemcpyHostToDevice));
  MGPBD_CUDA(cudaMemset(g_.p, 0, sizeof(float) * kNetParams));
  MGPBD_CUDA(cudaMemset(m_.p, 0, sizeof(float) * kNetParams));
  MGPBD_CUDA(cudaMemset(v_.p, 0, sizeof(float) * kNetParams));
  sync_params(nullptr);
  MGPBD_CUDA(cudaStreamSynchronize(nullptr));
}

void CoarseNet::sync_params(cudaStream_t s) {
  k_net_pack<<<ceil_div(4 * kNetF * kNetF, kT), kT, 0, s>>>(p_.p, wt_.p);
  MGPBD_CHECK_LAUNCH();
}

void CoarseNet::reset_adam(cudaStream_t s) {
  MGPBD_CUDA(cudaMemsetAsync(m_.p, 0, sizeof(float) * kNetParams, s));
  MGPBD_CUDA(cudaMemsetAsync(v_.p, 0, sizeof(float) * kNetParams, s));
  t_ = 0;
}

void CoarseNet::ensure(const NetGraph& g) {
  require(g.nnz >= g.n, MGPBD_EINVAL, "coarse net: nnz below the row count");
  if (g.nnz > ah_.n) ah_.alloc(g.nnz);
  const int32_t n = g.n;
  if (n <= cap_) return;
  const int64_t nf = (int64_t)n * kNetF;
  part_.alloc(kMaxReduceBlocks);
  sumsq_.alloc(2);
  u_.alloc(n);
  a1_.alloc(n);
  y_.alloc(n);
  e_.alloc(n);
  gy_.alloc(n);
  h3_.alloc(nf);
  gz_.alloc(nf);
  gself_.alloc(nf);
  q_.alloc(nf);
  h1_.alloc(nf);
  g1_.alloc(nf);
  h2_.alloc(nf);
  g2_.alloc(nf);
  feat_.alloc(n);
  wcap_.alloc(n);
  wv_.alloc(n);
  dw_.alloc(n);
  wpart_.alloc((int64_t)kWgradBlocks * kBigPart);
  cap_ = n;
}

void CoarseNet::run_forward(const NetGraph& g, const float* r, float* e, float* y_out, bool train,
                            float* cap_out, cudaStream_t s) {
  const int32_t n = g.n;
  const int rb = std::min(kMaxReduceBlocks, std::max(1, ceil_div(n, kT * 4)));
  k_net_sumsq<<<rb, kT, 0, s>>>(n, r, g.diag_inv, part_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_sum<<<1, kT, 0, s>>>(part_.p, rb, sumsq_.p, 0);
  MGPBD_CHECK_LAUNCH();
  k_net_l1<<<ceil_div(n, kT / 32), kT, 0, s>>>(g, r, sumsq_.p, p_.p, h1_.p, ah_.p, cap_out,
                                                train ? u_.p : nullptr, train ? a1_.p : nullptr);
  MGPBD_CHECK_LAUNCH();
  const int lb = ceil_div(n, kLayerRows);
  k_net_layer<false><<<lb, kLayerThreads, 0, s>>>(g, ah_.p, h1_.p, wt_.p, p_.p, kNetOffB2, h2_.p,
                                                  train ? g1_.p : nullptr, sumsq_.p, nullptr,
                                                  nullptr, nullptr);
  MGPBD_CHECK_LAUNCH();
  k_net_layer<true><<<lb, kLayerThreads, 0, s>>>(g, ah_.p, h2_.p, wt_.p + 2 * kNetF * kNetF, p_.p,
                                                 kNetOffB3, nullptr, train ? g2_.p : nullptr,
                                                 sumsq_.p, y_out ? y_out : (train ? y_.p : nullptr),
                                                 e, train ? h3_.p : nullptr);
  MGPBD_CHECK_LAUNCH();
}

void CoarseNet::weights(const NetGraph& g, float* w, cudaStream_t s) {
  require(g.n > 0, MGPBD_EINVAL, "coarse net: empty graph");
  ensure(g);
  k_net_feat<<<ceil_div(g.n, kT), kT, 0, s>>>(g.n, g.diag_inv, feat_.p);
  MGPBD_CHECK_LAUNCH();
  run_forward(g, feat_.p, e_.p, y_.p, false, wcap_.p, s);
  k_net_squash<<<ceil_div(g.n, kT), kT, 0, s>>>(g.n, y_.p, wcap_.p, w, nullptr);
  MGPBD_CHECK_LAUNCH();
}

void apply_coarse_weights(int32_t n, const float* w, const float* diag_inv, const float* r,
                          float* e, cudaStream_t s) {
  k_net_apply<<<ceil_div(n, kT), kT, 0, s>>>(n, w, diag_inv, r, e);
  MGPBD_CHECK_LAUNCH();
}

void CoarseNet::forward(const NetGraph& g, const float* r, float* e, cudaStream_t s) {
  require(g.n > 0, MGPBD_EINVAL, "coarse net: empty graph");
  ensure(g);
  run_forward(g, r, e, nullptr, false, nullptr, s);
}

// Gradients of every parameter from gy (output) and gz (head pre-activation
// gradient) of the activations stored by the last training forward.
void CoarseNet::backward_layers(const NetGraph& g, cudaStream_t s) {
  const int32_t n = g.n;
  const int wb = std::min(kWgradBlocks, std::max(1, ceil_div(n, 64)));
  const int rowb = ceil_div(n, kT / 32);
  k_net_wgrad_out<<<wb, kT, 0, s>>>(n, h3_.p, gy_.p, wpart_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_wsum<<<1, kT, 0, s>>>(wpart_.p, wb, kNetF + 1, g_.p + kNetOffWo);
  MGPBD_CHECK_LAUNCH();
  // layer 3
  k_net_wgrad_big<<<wb, kT, 0, s>>>(n, h2_.p, g2_.p, gz_.p, wpart_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_wsum<<<ceil_div(kBigPart, kT), kT, 0, s>>>(wpart_.p, wb, kBigPart, g_.p + kNetOffW3);
  MGPBD_CHECK_LAUNCH();
  k_net_xgrad<<<ceil_div(n, 32), 2 * kNetF, 0, s>>>(n, gz_.p, wt_.p + 2 * kNetF * kNetF,
                                                     gself_.p, q_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_hgrad<<<rowb, kT, 0, s>>>(g, ah_.p, gself_.p, q_.p, h2_.p, gz_.p);
  MGPBD_CHECK_LAUNCH();
  // layer 2
  k_net_wgrad_big<<<wb, kT, 0, s>>>(n, h1_.p, g1_.p, gz_.p, wpart_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_wsum<<<ceil_div(kBigPart, kT), kT, 0, s>>>(wpart_.p, wb, kBigPart, g_.p + kNetOffW2);
  MGPBD_CHECK_LAUNCH();
  k_net_xgrad<<<ceil_div(n, 32), 2 * kNetF, 0, s>>>(n, gz_.p, wt_.p, gself_.p, q_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_hgrad<<<rowb, kT, 0, s>>>(g, ah_.p, gself_.p, q_.p, h1_.p, gz_.p);
  MGPBD_CHECK_LAUNCH();
  // layer 1
  k_net_wgrad_l1<<<wb, kT, 0, s>>>(n, u_.p, a1_.p, gz_.p, wpart_.p);
  MGPBD_CHECK_LAUNCH();
  k_net_wsum<<<1, kT, 0, s>>>(wpart_.p, wb, 3 * kNetF, g_.p + kNetOffW1s);
  MGPBD_CHECK_LAUNCH();
}

void CoarseNet::loss_grad(const NetGraph& g, const float* samples, int32_t n_samples,
                          int32_t first, int32_t batch, double* loss_dev, int32_t mode,
                          cudaStream_t s) {
  require(g.n > 0 && n_samples > 0 && batch > 0 && first >= 0, MGPBD_EINVAL,
          "coarse net: empty graph or batch");
  require(mode == kNetModeWeights || mode == kNetModeField, MGPBD_EINVAL,
          "coarse net: unknown loss mode");
  const int32_t S = batch;
  ensure(g);
  const int32_t n = g.n;
  MGPBD_CUDA(cudaMemsetAsync(g_.p, 0, sizeof(float) * kNetParams, s));
  MGPBD_CUDA(cudaMemsetAsync(loss_dev, 0, sizeof(double), s));
  const float scale = (float)(1.0 / ((double)n * (double)S));
  const int ob = std::min(kMaxReduceBlocks, ceil_div(n, kT / 32));
  const int rb = std::min(kMaxReduceBlocks, std::max(1, ceil_div(n, kT * 4)));
  auto sample = [&](int32_t k) {
    return samples + (int64_t)((first + (int64_t)k) % n_samples) * n;
  };
  if (mode == kNetModeWeights) {
    k_net_feat<<<ceil_div(n, kT), kT, 0, s>>>(n, g.diag_inv, feat_.p);
    MGPBD_CHECK_LAUNCH();
    run_forward(g, feat_.p, e_.p, nullptr, true, wcap_.p, s);
    k_net_squash<<<ceil_div(n, kT), kT, 0, s>>>(n, y_.p, wcap_.p, wv_.p, dw_.p);
    MGPBD_CHECK_LAUNCH();
    MGPBD_CUDA(cudaMemsetAsync(gy_.p, 0, sizeof(float) * n, s));
    for (int32_t k = 0; k < S; ++k) {
      k_net_sumsq<<<rb, kT, 0, s>>>(n, sample(k), g.diag_inv, part_.p);
      MGPBD_CHECK_LAUNCH();
      k_net_sum<<<1, kT, 0, s>>>(part_.p, rb, sumsq_.p + 1, 0);
      MGPBD_CHECK_LAUNCH();
      k_net_wloss<<<ob, kT, 0, s>>>(g, ah_.p, wv_.p, dw_.p, sample(k), sumsq_.p + 1, scale,
                                    gy_.p, part_.p);
      MGPBD_CHECK_LAUNCH();
      k_net_sum<<<1, kT, 0, s>>>(part_.p, ob, loss_dev, 1);
      MGPBD_CHECK_LAUNCH();
    }
    k_net_head_bwd<<<ceil_div((int64_t)n * kNetF, kT), kT, 0, s>>>(n, gy_.p, h3_.p, p_.p, gz_.p);
    MGPBD_CHECK_LAUNCH();
    backward_layers(g, s);
    return;
  }
  for (int32_t k = 0; k < S; ++k) {
    run_forward(g, sample(k), e_.p, nullptr, true, nullptr, s);
    k_net_out_bwd<<<ob, kT, 0, s>>>(g, ah_.p, y_.p, u_.p, h3_.p, p_.p, scale, gy_.p, gz_.p,
                                    part_.p);
    MGPBD_CHECK_LAUNCH();
    k_net_sum<<<1, kT, 0, s>>>(part_.p, ob, loss_dev, 1);
    MGPBD_CHECK_LAUNCH();
    backward_layers(g, s);
  }
}

void CoarseNet::train(const NetGraph& g, const float* samples, int32_t n_samples, int32_t batch,
                      int32_t steps, float lr, double* losses_dev, cudaStream_t s) {
  require(steps >= 0, MGPBD_EINVAL, "coarse net: negative step count");
  for (int32_t k = 0; k < steps; ++k) {
    const int32_t first = (int32_t)(((int64_t)k * batch) % n_samples);
    loss_grad(g, samples, n_samples, first, batch, losses_dev + k, kNetModeWeights, s);
    adam(lr, 0.9f, 0.999f, 1e-8f, s);
  }
}

void CoarseNet::adam(float lr, float beta1, float beta2, float eps, cudaStream_t s) {
  ++t_;
  const float bc1 = (float)(1.0 - std::pow((double)beta1, (double)t_));
  const float bc2 = (float)(1.0 - std::pow((double)beta2, (double)t_));
  k_net_adam<<<ceil_div(kNetParams, kT), kT, 0, s>>>(p_.p, g_.p, m_.p, v_.p, kNetParams, lr,
                                                     beta1, beta2, eps, bc1, bc2);
  MGPBD_CHECK_LAUNCH();
  sync_params(s);
}

}  // namespace mgpbd
