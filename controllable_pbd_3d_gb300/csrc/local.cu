// Local XPBD (cons/deform3d.py:7-288) and Vertex Block Descent
// (cons/vbd.py:6-361) on the GPU.
//
// Layouts: positions and velocities (nv, 3) float32 as the caller's fields;
// t_i as int4 per tet; per-tet rest data as (nt, 3, 3) row-major inverse
// rest-shape matrices (Dm_inv / B) and (nt) volumes; VBD's vertex-tet
// adjacency as CSR with entries tet * 4 + local index, tets ascending
// (_build_vertex_tet_adjacency, cons/vbd.py:68-96).
//
// Arithmetic is float32 in the reference's operation order per element;
// the colour kernels are deterministic (no two threads of a colour touch the
// same vertex, fixed lane-reduction order), the XPBD default method is not
// (its position updates are atomic adds racing with other tets' reads, like
// the reference's parallel loop).
#include "local.cuh"

#include <algorithm>
#include <cmath>
#include <string>

#include "coloring.h"
#include "persist.cuh"

namespace mgpbd {

namespace {

constexpr int kLT = 256;  // threads per block
constexpr int kVL = 4;    // lanes per vertex in the VBD colour kernel
constexpr unsigned long long kSpinNs = 4000000000ull;  // grid barrier limit

// 3x3 helpers (row-major m[r][c]); determinant by the first column's
// cofactors, inverse = adjugate / det
__device__ __forceinline__ float det3(const float m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) -
         m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
         m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

__device__ __forceinline__ void inv3(const float m[3][3], float r[3][3]) {
  const float id = 1.0f / det3(m);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      r[j][i] = id * (m[(i + 1) % 3][(j + 1) % 3] * m[(i + 2) % 3][(j + 2) % 3] -
                      m[(i + 2) % 3][(j + 1) % 3] * m[(i + 1) % 3][(j + 2) % 3]);
}

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ float nsq3(const float a[3]) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }
__device__ __forceinline__ float dot3(const float a[3], const float b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// F = D B with D's columns x_k - x_4 (d[k][i] = (x_k - x_4)_i); column j of
// F is f[j][.]
__device__ __forceinline__ void deformation(const float p[4][3], const float B[3][3],
                                            float f[3][3]) {
  float d[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i) d[k][i] = p[k][i] - p[3][i];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) f[j][i] = d[0][i] * B[0][j] + d[1][i] * B[1][j] + d[2][i] * B[2][j];
}

// det of the matrix whose columns are f[0], f[1], f[2]
__device__ __forceinline__ float det_cols(const float f[3][3]) {
  float m[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) m[i][j] = f[j][i];
  return det3(m);
}

// rest shape of tet k: Dm (columns r_k - r_4), its inverse and |det| / 6
// (_precompute_rest_shape, cons/vbd.py:111-124; the B of
// cons/deform3d.py:75)
__global__ void k_rest_shape(const float* __restrict__ x_ref, const int4* __restrict__ t_i,
                             int32_t nt, float* __restrict__ dm_inv, float* __restrict__ vol) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int4 q = t_i[k];
    const int32_t v[4] = {q.x, q.y, q.z, q.w};
    float r[4][3];
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
      for (int c = 0; c < 3; ++c) r[l][c] = x_ref[3LL * v[l] + c];
    float dm[3][3], inv[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) dm[i][j] = r[j][i] - r[3][i];
    inv3(dm, inv);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) dm_inv[9 * k + 3 * i + j] = inv[i][j];
    if (vol) vol[k] = fabsf(det3(dm)) / 6.0f;
  }
}

// ---------------------------------------------------------------------------
// local XPBD: the coupled hydrostatic (det F - 1) and deviatoric
// (|F|^2 - 3) constraints of one tet (cons/deform3d.py:57-127)

struct XArgs {
  float* x;
  const float* invm;
  const int4* t_i;
  const float* t_m;
  const float* B;
  float* lh;
  float* ld;
  int32_t nt;
  float dt, ha, da;
};

// ATOMIC: positions read through L2 and updated with atomic adds (the
// parallel default method); otherwise plain read-modify-write in the
// reference's order (all hydrostatic updates, then all deviatoric ones)
template <bool ATOMIC>
__device__ __forceinline__ void xpbd_tet(const XArgs& a, int64_t k) {
  const int4 q = a.t_i[k];
  const int64_t vid[4] = {q.x, q.y, q.z, q.w};
  float p[4][3], w[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) {
#pragma unroll
    for (int c = 0; c < 3; ++c) p[l][c] = ATOMIC ? __ldcg(a.x + 3 * vid[l] + c) : a.x[3 * vid[l] + c];
    w[l] = a.invm[vid[l]];
  }
  float B[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) B[r][c] = a.B[9 * k + 3 * r + c];
  float f[3][3];
  deformation(p, B, f);

  const float CH = det_cols(f) - 1.0f;
  float cof[3][3];  // columns f2 x f3, f3 x f1, f1 x f2
  cross3(f[1], f[2], cof[0]);
  cross3(f[2], f[0], cof[1]);
  cross3(f[0], f[1], cof[2]);
  float gH[4][3], gD[4][3];  // gradients per vertex: columns of cof B^T and 2 F B^T
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      gH[j][i] = cof[0][i] * B[j][0] + cof[1][i] * B[j][1] + cof[2][i] * B[j][2];
      gD[j][i] = (2.0f * f[0][i]) * B[j][0] + (2.0f * f[1][i]) * B[j][1] +
                 (2.0f * f[2][i]) * B[j][2];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    gH[3][i] = -gH[0][i] - gH[1][i] - gH[2][i];
    gD[3][i] = -gD[0][i] - gD[1][i] - gD[2][i];
  }
  const float SH = w[0] * nsq3(gH[0]) + w[1] * nsq3(gH[1]) + w[2] * nsq3(gH[2]) + w[3] * nsq3(gH[3]);
  const float tm = a.t_m[k];
  const float aH = a.ha / (a.dt * a.dt * tm);
  float FF = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) FF += f[j][i] * f[j][i];
  const float CD = FF - 3.0f;
  const float SD = w[0] * nsq3(gD[0]) + w[1] * nsq3(gD[1]) + w[2] * nsq3(gD[2]) + w[3] * nsq3(gD[3]);
  const float aD = a.da / (a.dt * a.dt * tm);
  const float SDH = w[0] * dot3(gD[0], gH[0]) + w[1] * dot3(gD[1], gH[1]) +
                    w[2] * dot3(gD[2], gH[2]) + w[3] * dot3(gD[3], gH[3]);
  const float lH = a.lh[k], lD = a.ld[k];
  const float dH = (SDH * (CD + aD * lD) - (CH + aH * lH) * (aD + SD)) /
                   ((aH + SH) * (aD + SD) - SDH * SDH);
  const float dD = -(CD + aD * lD + SDH * dH) / (aD + SD);
#pragma unroll
  for (int l = 0; l < 4; ++l)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float u = w[l] * gH[l][c] * dH;
      if (ATOMIC) atomicAdd(a.x + 3 * vid[l] + c, u);
      else a.x[3 * vid[l] + c] = a.x[3 * vid[l] + c] + u;
    }
  a.lh[k] = lH + dH;
#pragma unroll
  for (int l = 0; l < 4; ++l)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float u = w[l] * gD[l][c] * dD;
      if (ATOMIC) atomicAdd(a.x + 3 * vid[l] + c, u);
      else a.x[3 * vid[l] + c] = a.x[3 * vid[l] + c] + u;
    }
  a.ld[k] = lD + dD;
}

// solve_cons (cons/deform3d.py:55-127): every tet at once
__global__ void __launch_bounds__(kLT) k_xpbd_all(XArgs a) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.nt;
       k += (int64_t)gridDim.x * blockDim.x)
    xpbd_tet<true>(a, k);
}

// solve_cons_gauss_seidel (:128-200): one tet at a time, in index order
__global__ void k_xpbd_serial(XArgs a, int32_t passes) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int32_t s = 0; s < passes; ++s)
    for (int64_t k = 0; k < a.nt; ++k) xpbd_tet<false>(a, k);
}

struct ColorArgs {
  const int32_t* order;
  const int32_t* off;
  int32_t n_colors;
  int32_t passes;
  GridSync* gs;
  int32_t* status;
};

// solve_cons_graph_coloring / solve_range (:210-288): the tets of one colour
// share no vertex; a grid barrier separates the colours
__global__ void __launch_bounds__(kLT) k_xpbd_color(XArgs a, ColorArgs c) {
  unsigned long long gen = 0;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int32_t s = 0; s < c.passes; ++s)
    for (int32_t col = 0; col < c.n_colors; ++col) {
      const int32_t b = c.off[col], e = c.off[col + 1];
      for (int64_t i = b + tid; i < e; i += stride) xpbd_tet<false>(a, c.order[i]);
      const bool last = s == c.passes - 1 && col == c.n_colors - 1;
      if (!last && !pdev::grid_sync(c.gs, c.status, kSpinNs, gen)) return;
    }
}

// ---------------------------------------------------------------------------
// VBD: one vertex's Newton step on its inertia + the Neo-Hookean-style
// energy of its incident tets (cons/vbd.py:186-266)

struct VArgs {
  float* x;
  const float* invm;
  const int4* t_i;
  const float* dm;
  const float* vol;
  const int32_t* adj_ptr;
  const int32_t* adj;
  const float* xt;
  const float* xo;
  float* xp;
  int32_t nv;
  float mu, lam, h2, dt, kd;
  int32_t keep_prev;
};

// force and Gauss-Newton Hessian (upper triangle 00 11 22 01 02 12) of one
// incident tet, added to f / H
__device__ __forceinline__ void vbd_entry(const VArgs& a, int32_t ent, float fo[3], float H[6]) {
  const int64_t tet = ent >> 2;
  const int l = ent & 3;
  const int4 q = a.t_i[tet];
  const int64_t vid[4] = {q.x, q.y, q.z, q.w};
  float p[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) p[k][c] = a.x[3 * vid[k] + c];
  float B[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) B[r][c] = a.dm[9 * tet + 3 * r + c];
  float f[3][3];
  deformation(p, B, f);
  const float J = det_cols(f);
  float cof[3][3];
  cross3(f[1], f[2], cof[0]);
  cross3(f[2], f[0], cof[1]);
  cross3(f[0], f[1], cof[2]);
  const float s = a.lam * (J - 1.0f);
  float b[3];
  if (l < 3) {
    b[0] = B[l][0];
    b[1] = B[l][1];
    b[2] = B[l][2];
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) b[c] = -(B[0][c] + B[1][c] + B[2][c]);
  }
  const float V0 = a.vol[tet];
  float qv[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    // P = mu F + lam (J - 1) cof F; f_e = -V0 (P b)
    const float pb = (a.mu * f[0][i] + s * cof[0][i]) * b[0] + (a.mu * f[1][i] + s * cof[1][i]) * b[1] +
                     (a.mu * f[2][i] + s * cof[2][i]) * b[2];
    fo[i] += -V0 * pb;
    qv[i] = cof[0][i] * b[0] + cof[1][i] * b[1] + cof[2][i] * b[2];
  }
  const float mb = a.mu * nsq3(b);
  H[0] += V0 * (mb + a.lam * (qv[0] * qv[0]));
  H[1] += V0 * (mb + a.lam * (qv[1] * qv[1]));
  H[2] += V0 * (mb + a.lam * (qv[2] * qv[2]));
  H[3] += V0 * (a.lam * (qv[0] * qv[1]));
  H[4] += V0 * (a.lam * (qv[0] * qv[2]));
  H[5] += V0 * (a.lam * (qv[1] * qv[2]));
}

// inertia, damping and the 3x3 solve of vertex vi from the summed tet
// terms; skipped (as the reference) when |det H| <= 1e-10
__device__ __forceinline__ void vbd_finish(const VArgs& a, int64_t vi, float w, const float fs[3],
                                           const float Hs[6]) {
  const float mi = 1.0f / w;
  const float mh = mi / a.h2;
  float x[3], f[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    x[c] = a.x[3 * vi + c];
    f[c] = mh * (a.xt[3 * vi + c] - x[c]) + fs[c];
  }
  if (a.keep_prev) {
#pragma unroll
    for (int c = 0; c < 3; ++c) a.xp[3 * vi + c] = x[c];
  }
  float H[3][3] = {{mh + Hs[0], Hs[3], Hs[4]}, {Hs[3], mh + Hs[1], Hs[5]}, {Hs[4], Hs[5], mh + Hs[2]}};
  if (a.kd > 0.0f) {
    const float kdt = a.kd / a.dt;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      f[c] -= kdt * (x[c] - a.xo[3 * vi + c]);
      H[c][c] += kdt;
    }
  }
  if (fabsf(det3(H)) > 1e-10f) {
    float inv[3][3];
    inv3(H, inv);
#pragma unroll
    for (int i = 0; i < 3; ++i)
      a.x[3 * vi + i] = x[i] + (inv[i][0] * f[0] + inv[i][1] * f[1] + inv[i][2] * f[2]);
  }
}

// sum of 9 values over groups of W lanes (fixed xor tree; all 32 lanes call)
template <int W>
__device__ __forceinline__ void group_sum(float f[3], float H[6]) {
#pragma unroll
  for (int sh = W / 2; sh > 0; sh >>= 1) {
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] += __shfl_xor_sync(0xffffffffu, f[c], sh, W);
#pragma unroll
    for (int c = 0; c < 6; ++c) H[c] += __shfl_xor_sync(0xffffffffu, H[c], sh, W);
  }
}

// _apply_chebyshev (cons/vbd.py:180-184) for vertices [t0, n) strided
__device__ __forceinline__ void vbd_chebyshev(const VArgs& a, float om, int64_t t0, int64_t step) {
  for (int64_t v = t0; v < a.nv; v += step) {
    if (a.invm[v] > 0.0f) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float xv = a.x[3 * v + c];
        a.x[3 * v + c] = xv + om * (xv - a.xp[3 * v + c]);
      }
    }
  }
}

// solve with method 'serial' (cons/vbd.py:134-160, 186-266): one block;
// warp 0 walks the vertices in index order, its 32 lanes splitting each
// vertex's incident tets
__global__ void k_vbd_serial(VArgs a, const float* __restrict__ om, int32_t n_iter, float rho) {
  const int lane = threadIdx.x & 31;
  for (int32_t n = 0; n < n_iter; ++n) {
    if (threadIdx.x < 32) {
      for (int64_t vi = 0; vi < a.nv; ++vi) {
        const float w = a.invm[vi];
        if (w == 0.0f) continue;
        float f[3] = {0.f, 0.f, 0.f}, H[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int32_t j = a.adj_ptr[vi] + lane; j < a.adj_ptr[vi + 1]; j += 32) vbd_entry(a, a.adj[j], f, H);
        group_sum<32>(f, H);
        if (lane == 0) vbd_finish(a, vi, w, f, H);
        __syncwarp();
      }
    }
    __syncthreads();
    if (rho > 0.0f && n >= 1) {
      vbd_chebyshev(a, om[n], threadIdx.x, blockDim.x);
      __syncthreads();
    }
  }
}

struct VColorArgs {
  const int32_t* order;
  const int32_t* off;
  int32_t n_colors;
  int32_t n_iter;
  float rho;
  const float* om;
  GridSync* gs;
  int32_t* status;
};

// solve with method 'color' (_solve_vertex_range, cons/vbd.py:267-361): the
// vertices of one colour share no tet; kVL lanes per vertex; grid barriers
// between colours and around the Chebyshev step
__global__ void __launch_bounds__(kLT) k_vbd_color(VArgs a, VColorArgs c) {
  unsigned long long gen = 0;
  constexpr int kPerWarp = 32 / kVL;
  const int lane = threadIdx.x & 31;
  const int sub = lane / kVL, gl = lane % kVL;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int32_t n = 0; n < c.n_iter; ++n) {
    const bool cheb = c.rho > 0.0f && n >= 1;
    for (int32_t col = 0; col < c.n_colors; ++col) {
      const int32_t b = c.off[col], e = c.off[col + 1];
      for (int64_t base = b + warp * kPerWarp; base < e; base += nwarps * kPerWarp) {
        const int64_t idx = base + sub;
        int64_t vi = 0;
        float w = 0.0f;
        if (idx < e) {
          vi = c.order[idx];
          w = a.invm[vi];
        }
        float f[3] = {0.f, 0.f, 0.f}, H[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (w != 0.0f)
          for (int32_t j = a.adj_ptr[vi] + gl; j < a.adj_ptr[vi + 1]; j += kVL) vbd_entry(a, a.adj[j], f, H);
        group_sum<kVL>(f, H);
        if (gl == 0 && w != 0.0f) vbd_finish(a, vi, w, f, H);
      }
      const bool last = n == c.n_iter - 1 && col == c.n_colors - 1 && !cheb;
      if (!last && !pdev::grid_sync(c.gs, c.status, kSpinNs, gen)) return;
    }
    if (cheb) {
      vbd_chebyshev(a, c.om[n], tid, stride);
      if (n != c.n_iter - 1 && !pdev::grid_sync(c.gs, c.status, kSpinNs, gen)) return;
    }
  }
}

// make_prediction (cons/vbd.py:125-132)
__global__ void k_vbd_predict(float* __restrict__ x, const float* __restrict__ v,
                              float* __restrict__ xo, float* __restrict__ xt, int64_t n3, float dt,
                              float gx, float gy, float gz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(i % 3);
    const float g = c == 0 ? gx : (c == 1 ? gy : gz);
    const float p = x[i];
    xo[i] = p;
    const float t = p + v[i] * dt + g * dt * dt;
    xt[i] = t;
    x[i] = t;
  }
}

// update_vel (cons/vbd.py:161-166)
__global__ void k_vbd_vel(const float* __restrict__ x, const float* __restrict__ xo,
                          float* __restrict__ v, int64_t n3, float damp, float dt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = damp * (x[i] - xo[i]) / dt;
}

int blocks_for(int64_t n) {
  const int64_t g = (n + kLT - 1) / kLT;
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(g, 4096)));
}

// one block per SM (cooperative launches; fewer blocks keep the barrier
// cheap, and a colour rarely has more elements than 152 x 256 threads)
int coop_grid(const void* fn) {
  int dev = 0, sms = 0, occ = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kLT, 0));
  require(occ >= 1, MGPBD_ECUDA, "local solver kernel cannot be resident");
  return sms;
}

// host copy of t_i with ids validated
std::vector<int32_t> host_tets(const int32_t* t_i, int32_t nt, int32_t nv) {
  std::vector<int32_t> h(static_cast<size_t>(nt) * 4);
  MGPBD_CUDA(cudaMemcpy(h.data(), t_i, sizeof(int32_t) * h.size(), cudaMemcpyDeviceToHost));
  for (int32_t v : h) require(v >= 0 && v < nv, MGPBD_EINVAL, "tet vertex id out of range");
  return h;
}

void upload(DevBuf<int32_t>& d, const std::vector<int32_t>& h, cudaStream_t s) {
  d.alloc(std::max<int64_t>(1, static_cast<int64_t>(h.size())));
  if (!h.empty())
    MGPBD_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(int32_t) * h.size(), cudaMemcpyHostToDevice, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

// ---------------------------------------------------------------------------

LazyStatus::~LazyStatus() {
  if (ev_) cudaEventDestroy(ev_);
  if (host_) cudaFreeHost(host_);
}

void LazyStatus::record(const int32_t* dev, cudaStream_t s) {
  if (!host_) {
    MGPBD_CUDA(cudaMallocHost(&host_, sizeof(int32_t)));
    *host_ = 0;
    MGPBD_CUDA(cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming));
  }
  MGPBD_CUDA(cudaMemcpyAsync(host_, dev, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaEventRecord(ev_, s));
  pending_ = true;
}

void LazyStatus::check(const char* what) {
  if (!pending_) return;
  const cudaError_t e = cudaEventQuery(ev_);
  if (e == cudaErrorNotReady) return;
  MGPBD_CUDA(e);
  pending_ = false;
  if (static_cast<uint32_t>(*host_) & MGPBD_STATUS_SYNC_TIMEOUT)
    throw Error(MGPBD_ECUDA, std::string(what) + ": a grid barrier wait timed out");
}

void LazyStatus::wait(const char* what) {
  if (!pending_) return;
  MGPBD_CUDA(cudaEventSynchronize(ev_));
  check(what);
}

Xpbd::Xpbd(const mgpbd_xpbd_params& p) : p_(p) {
  require(p.dt > 0.0f, MGPBD_EINVAL, "xpbd: dt must be positive");
  require(p.method >= MGPBD_XPBD_DEFAULT && p.method <= MGPBD_XPBD_GRAPH_COLORING, MGPBD_EINVAL,
          "xpbd: unknown method");
}

void Xpbd::set_mesh(float* x, const float* x_ref, const float* invm, const int32_t* t_i,
                    const float* t_m, int32_t nv, int32_t nt) {
  require(x && x_ref && invm && t_i && t_m, MGPBD_EINVAL, "xpbd: null mesh pointer");
  require(nv > 0 && nt > 0, MGPBD_EINVAL, "xpbd: empty mesh");
  require(static_cast<int64_t>(nt) * 4 < INT32_MAX, MGPBD_ERANGE, "xpbd: too many tets");
  require(reinterpret_cast<uintptr_t>(t_i) % 16 == 0, MGPBD_EINVAL, "xpbd: t_i must be 16-byte aligned");
  const std::vector<int32_t> ht = host_tets(t_i, nt, nv);
  x_ = x;
  invm_ = invm;
  t_i_ = t_i;
  t_m_ = t_m;
  nv_ = nv;
  nt_ = nt;
  cudaStream_t s = stream_;
  B_.alloc(9LL * nt);
  lam_h_.alloc(nt);
  lam_d_.alloc(nt);
  MGPBD_CUDA(cudaMemsetAsync(lam_h_.p, 0, sizeof(float) * nt, s));
  MGPBD_CUDA(cudaMemsetAsync(lam_d_.p, 0, sizeof(float) * nt, s));
  k_rest_shape<<<blocks_for(nt), kLT, 0, s>>>(x_ref, reinterpret_cast<const int4*>(t_i), nt, B_.p,
                                              nullptr);
  MGPBD_CHECK_LAUNCH();
  status_.alloc(1);
  MGPBD_CUDA(cudaMemsetAsync(status_.p, 0, sizeof(int32_t), s));
  n_colors_ = 0;
  if (p_.method == MGPBD_XPBD_GRAPH_COLORING) {
    const Coloring col = color_elements(ht.data(), nt, 4, nv);
    n_colors_ = col.n_colors;
    upload(order_, col.ordered, s);
    upload(offsets_, col.offsets, s);
    gs_.alloc(1);
    grid_ = coop_grid(reinterpret_cast<const void*>(k_xpbd_color));
  }
  MGPBD_CUDA(cudaStreamSynchronize(s));
}

void Xpbd::preupdate() {
  require(x_ != nullptr, MGPBD_ESTATE, "xpbd: set_mesh has not been called");
  MGPBD_CUDA(cudaMemsetAsync(lam_h_.p, 0, sizeof(float) * nt_, stream_));
  MGPBD_CUDA(cudaMemsetAsync(lam_d_.p, 0, sizeof(float) * nt_, stream_));
}

void Xpbd::update(int32_t passes) {
  require(x_ != nullptr, MGPBD_ESTATE, "xpbd: set_mesh has not been called");
  require(passes >= 0, MGPBD_EINVAL, "xpbd: negative pass count");
  lazy_.check("xpbd colour kernel");
  if (passes == 0) return;
  XArgs a;
  a.x = x_;
  a.invm = invm_;
  a.t_i = reinterpret_cast<const int4*>(t_i_);
  a.t_m = t_m_;
  a.B = B_.p;
  a.lh = lam_h_.p;
  a.ld = lam_d_.p;
  a.nt = nt_;
  a.dt = p_.dt;
  a.ha = p_.hydro_alpha;
  a.da = p_.devia_alpha;
  cudaStream_t s = stream_;
  if (p_.method == MGPBD_XPBD_DEFAULT) {
    for (int32_t i = 0; i < passes; ++i) {
      k_xpbd_all<<<blocks_for(nt_), kLT, 0, s>>>(a);
      MGPBD_CHECK_LAUNCH();
    }
    return;
  }
  if (p_.method == MGPBD_XPBD_GAUSS_SEIDEL) {
    k_xpbd_serial<<<1, 32, 0, s>>>(a, passes);
    MGPBD_CHECK_LAUNCH();
    return;
  }
  ColorArgs c;
  c.order = order_.p;
  c.off = offsets_.p;
  c.n_colors = n_colors_;
  c.passes = passes;
  c.gs = gs_.p;
  c.status = status_.p;
  MGPBD_CUDA(cudaMemsetAsync(gs_.p, 0, sizeof(GridSync), s));
  void* args[] = {&a, &c};
  MGPBD_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_xpbd_color), dim3(grid_),
                                         dim3(kLT), args, 0, s));
  MGPBD_CHECK_LAUNCH();
  lazy_.record(status_.p, s);
}

// ---------------------------------------------------------------------------

Vbd::Vbd(const mgpbd_vbd_params& p) : p_(p) {
  require(p.dt > 0.0f, MGPBD_EINVAL, "vbd: dt must be positive");
  require(p.method == MGPBD_VBD_SERIAL || p.method == MGPBD_VBD_COLOR, MGPBD_EINVAL,
          "vbd: unknown method");
  require(p.n_iterations >= 0, MGPBD_EINVAL, "vbd: negative iteration count");
  // Lame parameters in double, then float32 (cons/vbd.py:41-46)
  const double E = p.youngs_modulus, nu = p.poissons_ratio;
  mu_ = static_cast<float>(E / (2.0 * (1.0 + nu)));
  lam_ = static_cast<float>(E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
  // the omega sequence of solve (cons/vbd.py:141-151), in double like the
  // Python loop, passed to the kernel as float32
  omegas_.assign(static_cast<size_t>(p.n_iterations), 1.0f);
  double om = 1.0;
  const double r = p.rho;
  for (int32_t n = 0; n < p.n_iterations; ++n) {
    if (r > 0.0 && n >= 1) {
      om = n == 1 ? 2.0 / (2.0 - r * r) : 4.0 / (4.0 - r * r * om);
    }
    omegas_[n] = static_cast<float>(om);
  }
}

void Vbd::set_mesh(float* x, const float* x_ref, const float* invm, const int32_t* t_i, int32_t nv,
                   int32_t nt) {
  require(x && x_ref && invm && t_i, MGPBD_EINVAL, "vbd: null mesh pointer");
  require(nv > 0 && nt > 0, MGPBD_EINVAL, "vbd: empty mesh");
  require(static_cast<int64_t>(nt) * 4 < INT32_MAX, MGPBD_ERANGE, "vbd: too many tets");
  require(reinterpret_cast<uintptr_t>(t_i) % 16 == 0, MGPBD_EINVAL, "vbd: t_i must be 16-byte aligned");
  const std::vector<int32_t> ht = host_tets(t_i, nt, nv);
  x_ = x;
  x_ref_ = x_ref;
  invm_ = invm;
  t_i_ = t_i;
  nv_ = nv;
  nt_ = nt;
  inited_ = false;
  cudaStream_t s = stream_;
  // vertex -> (tet, local) entries, tets ascending (cons/vbd.py:68-96)
  std::vector<int32_t> ptr(static_cast<size_t>(nv) + 1, 0), ent(ht.size());
  for (int32_t v : ht) ptr[v + 1] += 1;
  for (int32_t v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int32_t t = 0; t < nt; ++t)
    for (int l = 0; l < 4; ++l) ent[fill[ht[4 * static_cast<size_t>(t) + l]]++] = 4 * t + l;
  upload(adj_ptr_, ptr, s);
  upload(adj_, ent, s);
  v_.alloc(3LL * nv);
  x_old_.alloc(3LL * nv);
  x_tilde_.alloc(3LL * nv);
  x_prev_.alloc(3LL * nv);
  dm_inv_.alloc(9LL * nt);
  vol_.alloc(nt);
  MGPBD_CUDA(cudaMemsetAsync(v_.p, 0, sizeof(float) * 3 * nv, s));
  MGPBD_CUDA(cudaMemsetAsync(x_old_.p, 0, sizeof(float) * 3 * nv, s));
  MGPBD_CUDA(cudaMemsetAsync(x_tilde_.p, 0, sizeof(float) * 3 * nv, s));
  MGPBD_CUDA(cudaMemsetAsync(x_prev_.p, 0, sizeof(float) * 3 * nv, s));
  om_.alloc(std::max<int64_t>(1, static_cast<int64_t>(omegas_.size())));
  if (!omegas_.empty())
    MGPBD_CUDA(cudaMemcpyAsync(om_.p, omegas_.data(), sizeof(float) * omegas_.size(),
                               cudaMemcpyHostToDevice, s));
  status_.alloc(1);
  MGPBD_CUDA(cudaMemsetAsync(status_.p, 0, sizeof(int32_t), s));
  n_colors_ = 0;
  if (p_.method == MGPBD_VBD_COLOR) {
    const Coloring col = color_vertices(ht.data(), nt, 4, nv);
    n_colors_ = col.n_colors;
    upload(order_, col.ordered, s);
    upload(offsets_, col.offsets, s);
    gs_.alloc(1);
    grid_ = coop_grid(reinterpret_cast<const void*>(k_vbd_color));
  }
  MGPBD_CUDA(cudaStreamSynchronize(s));
}

void Vbd::init() {
  require(x_ != nullptr, MGPBD_ESTATE, "vbd: set_mesh has not been called");
  k_rest_shape<<<blocks_for(nt_), kLT, 0, stream_>>>(x_ref_, reinterpret_cast<const int4*>(t_i_),
                                                     nt_, dm_inv_.p, vol_.p);
  MGPBD_CHECK_LAUNCH();
  inited_ = true;
}

void Vbd::make_prediction() {
  require(inited_, MGPBD_ESTATE, "vbd: init has not been called");
  const int64_t n3 = 3LL * nv_;
  k_vbd_predict<<<blocks_for(n3), kLT, 0, stream_>>>(x_, v_.p, x_old_.p, x_tilde_.p, n3, p_.dt,
                                                     p_.gravity[0], p_.gravity[1], p_.gravity[2]);
  MGPBD_CHECK_LAUNCH();
}

void Vbd::update_vel() {
  require(inited_, MGPBD_ESTATE, "vbd: init has not been called");
  const int64_t n3 = 3LL * nv_;
  k_vbd_vel<<<blocks_for(n3), kLT, 0, stream_>>>(x_, x_old_.p, v_.p, n3, p_.damp, p_.dt);
  MGPBD_CHECK_LAUNCH();
}

void Vbd::solve() {
  require(inited_, MGPBD_ESTATE, "vbd: init has not been called");
  lazy_.check("vbd colour kernel");
  if (p_.n_iterations == 0) return;
  VArgs a;
  a.x = x_;
  a.invm = invm_;
  a.t_i = reinterpret_cast<const int4*>(t_i_);
  a.dm = dm_inv_.p;
  a.vol = vol_.p;
  a.adj_ptr = adj_ptr_.p;
  a.adj = adj_.p;
  a.xt = x_tilde_.p;
  a.xo = x_old_.p;
  a.xp = x_prev_.p;
  a.nv = nv_;
  a.mu = mu_;
  a.lam = lam_;
  a.dt = p_.dt;
  a.h2 = p_.dt * p_.dt;
  a.kd = p_.damping;
  a.keep_prev = p_.rho > 0.0f ? 1 : 0;
  cudaStream_t s = stream_;
  if (p_.method == MGPBD_VBD_SERIAL) {
    k_vbd_serial<<<1, kLT, 0, s>>>(a, om_.p, p_.n_iterations, p_.rho);
    MGPBD_CHECK_LAUNCH();
    return;
  }
  VColorArgs c;
  c.order = order_.p;
  c.off = offsets_.p;
  c.n_colors = n_colors_;
  c.n_iter = p_.n_iterations;
  c.rho = p_.rho;
  c.om = om_.p;
  c.gs = gs_.p;
  c.status = status_.p;
  MGPBD_CUDA(cudaMemsetAsync(gs_.p, 0, sizeof(GridSync), s));
  void* args[] = {&a, &c};
  MGPBD_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_vbd_color), dim3(grid_),
                                         dim3(kLT), args, 0, s));
  MGPBD_CHECK_LAUNCH();
  lazy_.record(status_.p, s);
}

void* Vbd::field(int32_t f, int64_t* count) {
  switch (f) {
    case MGPBD_VBD_FIELD_V: *count = 3LL * nv_; return v_.p;
    case MGPBD_VBD_FIELD_X_OLD: *count = 3LL * nv_; return x_old_.p;
    case MGPBD_VBD_FIELD_X_TILDE: *count = 3LL * nv_; return x_tilde_.p;
    case MGPBD_VBD_FIELD_DM_INV: *count = 9LL * nt_; return dm_inv_.p;
    case MGPBD_VBD_FIELD_REST_VOL: *count = nt_; return vol_.p;
    default: throw Error(MGPBD_EINVAL, "vbd: unknown field");
  }
}

}  // namespace mgpbd
