// The MGPBD linear solve in its primal (vertex-space) form, as ONE
// cooperative persistent kernel per solve.
//
// The Newton system of the dual step is A dlam = b with A = alpha~ + J W J^T
// (one row per tet constraint).  By the Woodbury identity, restricted to the
// free vertices (w_v > 0),
//
//   dlam = alpha~^-1 (b - J y),   K y = J^T alpha~^-1 b,
//   K = W^-1 + J^T alpha~^-1 J    (3 nv x 3 nv, symmetric positive definite)
//
// and y is exactly the position update W J^T dlam.  A's spectrum carries a
// cluster at alpha~ (the null space of J^T, nt > 3 nv) on top of K's; CG on K
// needs about half the operator applications of CG on A at the same
// tolerance.  K is applied matrix-free from the same per-tet gradients as A,
// in the opposite phase order: tet phase s_t = (J v)_t / alpha~_t, vertex
// phase (K v)_v = m_v v_v + sum_{t incident to v} s_t g_{t,v}.
//
// The stopping test is the reference's: the dual residual |b - A dlam| of
// the dlam the current y gives, which is exactly |J W r_K| for the primal
// residual r_K; it is evaluated in the first tet phase of every iteration.
//
// Preconditioner: 3x3 block Jacobi (B_v = m_v I + sum_t g_{t,v} g_{t,v}^T /
// alpha~_t, inverted per vertex) inside a Chebyshev polynomial of degree k
// on [lambda_max * cheb_lo, 1.02 lambda_max] of B^-1 K.  lambda_max comes
// from the Lanczos tridiagonal of the first kBoot block-Jacobi PCG
// iterations (T_jj = 1/a_j + b_{j-1}/a_{j-1}, T_{j,j+1} = sqrt(b_j)/a_j;
// Saad, "Iterative Methods for Sparse Linear Systems", 2nd ed., sec. 6.7.3),
// computed in the kernel; CG then restarts from that iterate with the
// polynomial preconditioner.  No host round trip within a solve.
//
// Work split, staging, barriers and reductions as in jcg.cu.
#include <algorithm>
#include <cmath>

#include "common.h"
#include "jform.cuh"
#include "jform_dev.cuh"
#include "persist.cuh"

namespace mgpbd {

namespace {

using namespace jdev;
using namespace pdev;

constexpr int kPT = 576;  // threads per block, one block per SM
constexpr int kTB = 4;    // tets a thread handles per round of a tet phase
constexpr int kVS = 4;    // lanes per vertex in a vertex phase
constexpr int kVE = 6;    // entries a lane gathers per vertex and round
constexpr int kVB = 4;    // vertices a lane group handles per round
constexpr int kBoot = 24; // block-Jacobi PCG iterations that estimate lambda_max

struct QArgs {
  int32_t nt, nv;
  int32_t n4;          // length constraints from here on (compact in gE, qE)
  const float4* gE;    // their gradient n (slot 1 is -n)
  const int2* qE;      // their two vertices
  const int4* t_i;
  const float4* gradC;  // the 12 gradient entries as three planes of nt float4
  const float* alpha;   // alpha~
  const float* invm;
  const int32_t* inc_ptr;
  const float4* gV;  // vertex-major (gradient, tet id)
  const float* b;
  float* dlam;
  // vertex vectors, xyz used; r.w holds w_v (for the dual residual)
  float4 *y, *yc, *r, *z, *d, *p, *q, *rhs, *bi0, *bi1;
  float* s;          // tet scratch: (J v)_t / alpha~_t
  double* partials;  // 4 slots of gridDim.x
  GridSync* gs;
  CgState* st;
  const int32_t* part_v;
  const int32_t* part_t;
  int32_t emax, tmax, vmax;
  double tol_abs, tol_rel;
  int32_t maxiter, degree;
  float cheb_lo;
  int32_t stall_its;  // > 0: stop once the dual residual has not fallen by
                      // 10 % for this many iterations
  double max_amp;     // > 0: decline (stop at once, flags = 1) when the dual
                      // residual of the start exceeds max_amp |b|
  unsigned long long spin_ns;
};

struct Own {
  int64_t tbeg, tend, tstep;  // this thread's tets
  int64_t vbeg, vend, vstep;  // this thread's vertices in vertex-local loops
  int32_t tb0, vb0, nvb;      // staged: block ranges
  const float4* e;
  const int4* q;
  const int32_t* off;
  const float* w;
};

// thread-0 state of the solve (identical in every block)
struct Ctl {
  double bb, tol2, rz, pap, alpha, beta, rres, best, amp0;
  int32_t declined;
  int32_t since;  // iterations since the dual residual last fell by 10 %
  double ca[kBoot], cb[kBoot];  // bootstrap CG coefficients
  float c1[kMaxCheb], c2[kMaxCheb];
  float inv_theta, al, be;
  int32_t iters, nboot, stop;
  uint32_t status;
};

__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// z = B^-1 v, B^-1 symmetric as (i0 i1 i2 i3) (i4 i5 . .):
// [[i0 i1 i2] [i1 i3 i4] [i2 i4 i5]]
__device__ __forceinline__ float3 binv_apply(float4 i0, float4 i1, float3 v) {
  return make_float3(i0.x * v.x + i0.y * v.y + i0.z * v.z, i0.y * v.x + i0.w * v.y + i1.x * v.z,
                     i0.z * v.x + i1.x * v.y + i1.y * v.z);
}

__device__ __forceinline__ float4 p4(float3 v, float w = 0.0f) { return make_float4(v.x, v.y, v.z, w); }

// sum_l g_{t,l} . v_{q_l}
__device__ __forceinline__ float gdot(const float4 g0, const float4 g1, const float4 g2, float3 v0,
                                      float3 v1, float3 v2, float3 v3) {
  return (g0.x * v0.x + g0.y * v0.y + g0.z * v0.z) + (g0.w * v1.x + g1.x * v1.y + g1.y * v1.z) +
         (g1.z * v2.x + g1.w * v2.y + g2.x * v2.z) + (g2.y * v3.x + g2.z * v3.y + g2.w * v3.z);
}

template <bool STAGED>
__device__ __forceinline__ int4 tet_q(const QArgs& a, const Own& o, int64_t t) {
  if (STAGED) return o.q[t - o.tb0];
  return a.t_i[t];
}

// Tet phase.  MODE kTZ: s = J z / alpha~.  kT1: s = J (z + beta p) / alpha~
// and the squared dual residual sum_t (J W r)_t^2 into *acc.  kTY: s = J y /
// alpha~.  kTFinal: dlam = (b - J y) / alpha~.
enum TMode { kTZ = 0, kT1 = 1, kTY = 2, kTFinal = 3 };

template <int MODE, bool STAGED>
__device__ __forceinline__ void tphase(const QArgs& a, const Own& o, float beta, float* acc) {
  const float4* V = MODE == kTZ || MODE == kT1 ? a.z : a.y;
  for (int64_t tb = o.tbeg; tb < o.tend; tb += kTB * o.tstep) {
    float y[kTB], e[kTB];
#pragma unroll
    for (int i = 0; i < kTB; ++i) {
      const int64_t t = tb + i * o.tstep;
      y[i] = 0.0f;
      e[i] = 0.0f;
      if (!STAGED && t < o.tend && t >= a.n4) {
        // length constraint: two vertices, gradients n and -n
        const int2 qe = __ldg(a.qE + (t - a.n4));
        const float3 n = f3(__ldg(a.gE + (t - a.n4)));
        float3 v0 = f3(V[qe.x]), v1 = f3(V[qe.y]);
        if (MODE == kT1) {
          const float3 p0 = f3(a.p[qe.x]), p1 = f3(a.p[qe.y]);
          v0 = make_float3(v0.x + beta * p0.x, v0.y + beta * p0.y, v0.z + beta * p0.z);
          v1 = make_float3(v1.x + beta * p1.x, v1.y + beta * p1.y, v1.z + beta * p1.z);
          const float4 r0 = a.r[qe.x], r1 = a.r[qe.y];
          e[i] = dot3(n, make_float3(r0.w * r0.x, r0.w * r0.y, r0.w * r0.z)) -
                 dot3(n, make_float3(r1.w * r1.x, r1.w * r1.y, r1.w * r1.z));
        }
        y[i] = dot3(n, v0) - dot3(n, v1);
      } else if (t < o.tend) {
        const int4 q = tet_q<STAGED>(a, o, t);
        const float4 g0 = __ldg(a.gradC + t), g1 = __ldg(a.gradC + a.nt + t),
                     g2 = __ldg(a.gradC + 2LL * a.nt + t);
        float3 v0 = f3(V[q.x]), v1 = f3(V[q.y]), v2 = f3(V[q.z]), v3 = f3(V[q.w]);
        if (MODE == kT1) {
          const float3 p0 = f3(a.p[q.x]), p1 = f3(a.p[q.y]), p2 = f3(a.p[q.z]), p3 = f3(a.p[q.w]);
          v0 = make_float3(v0.x + beta * p0.x, v0.y + beta * p0.y, v0.z + beta * p0.z);
          v1 = make_float3(v1.x + beta * p1.x, v1.y + beta * p1.y, v1.z + beta * p1.z);
          v2 = make_float3(v2.x + beta * p2.x, v2.y + beta * p2.y, v2.z + beta * p2.z);
          v3 = make_float3(v3.x + beta * p3.x, v3.y + beta * p3.y, v3.z + beta * p3.z);
          const float4 r0 = a.r[q.x], r1 = a.r[q.y], r2 = a.r[q.z], r3 = a.r[q.w];
          e[i] = gdot(g0, g1, g2, make_float3(r0.w * r0.x, r0.w * r0.y, r0.w * r0.z),
                      make_float3(r1.w * r1.x, r1.w * r1.y, r1.w * r1.z),
                      make_float3(r2.w * r2.x, r2.w * r2.y, r2.w * r2.z),
                      make_float3(r3.w * r3.x, r3.w * r3.y, r3.w * r3.z));
        }
        y[i] = gdot(g0, g1, g2, v0, v1, v2, v3);
      }
    }
#pragma unroll
    for (int i = 0; i < kTB; ++i) {
      const int64_t t = tb + i * o.tstep;
      if (t < o.tend) {
        const float at = __ldg(a.alpha + t);
        if (MODE == kTFinal) {
          a.dlam[t] = (a.b[t] - y[i]) / at;
        } else {
          a.s[t] = y[i] / at;
        }
        if (MODE == kT1) *acc += e[i] * e[i];
      }
    }
  }
}

// Vertex phase core: for the lane group's vertices of each round, sum
// s_t g_{t,v} over the incident entries, then lane 0 calls
// epi(v, sum, w_v) for every free vertex.  All gathers of a round are
// issued before any is consumed.
template <bool STAGED, class Epi>
__device__ __forceinline__ void vphase(const QArgs& a, const Own& o, Epi&& epi) {
  const int lane = threadIdx.x % kVS;
  int64_t gidx, ngroups, nloop;
  if (STAGED) {
    gidx = threadIdx.x / kVS;
    ngroups = blockDim.x / kVS;
    nloop = o.nvb;
  } else {
    gidx = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kVS;
    ngroups = (int64_t)gridDim.x * blockDim.x / kVS;
    nloop = a.nv;
  }
  for (int64_t base = 0; base < nloop; base += kVB * ngroups) {
    int32_t k0[kVB], k1[kVB];
    float wv[kVB];
#pragma unroll
    for (int i = 0; i < kVB; ++i) {
      const int64_t lv = base + gidx + i * ngroups;
      k0[i] = k1[i] = 0;
      wv[i] = 0.0f;
      if (lv < nloop) {
        if (STAGED) {
          wv[i] = o.w[lv];
          if (wv[i] != 0.0f) {
            k0[i] = o.off[lv];
            k1[i] = o.off[lv + 1] - 1;
          }
        } else {
          wv[i] = a.invm[lv];
          if (wv[i] != 0.0f) {
            k0[i] = a.inc_ptr[lv];
            k1[i] = a.inc_ptr[lv + 1];
          }
        }
      }
    }
    float xs[kVB][kVE];
#pragma unroll
    for (int i = 0; i < kVB; ++i) {
#pragma unroll
      for (int c = 0; c < kVE; ++c) {
        const int32_t k = k0[i] + lane + kVS * c;
        float xt = 0.0f;
        if (k < k1[i]) {
          const float tw = STAGED ? o.e[k].w : __ldg(&a.gV[k].w);
          xt = a.s[__float_as_int(tw)];
        }
        xs[i][c] = xt;
      }
    }
#pragma unroll
    for (int i = 0; i < kVB; ++i) {
      float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
      for (int c = 0; c < kVE; ++c) {
        const int32_t k = k0[i] + lane + kVS * c;
        if (k < k1[i]) {
          const float4 g = STAGED ? o.e[k] : __ldg(a.gV + k);
          ax += xs[i][c] * g.x;
          ay += xs[i][c] * g.y;
          az += xs[i][c] * g.z;
        }
      }
      for (int32_t k = k0[i] + lane + kVS * kVE; k < k1[i]; k += kVS) {
        const float4 g = STAGED ? o.e[k] : __ldg(a.gV + k);
        const float xt = a.s[__float_as_int(g.w)];
        ax += xt * g.x;
        ay += xt * g.y;
        az += xt * g.z;
      }
#pragma unroll
      for (int sh = kVS / 2; sh > 0; sh >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, sh, kVS);
        ay += __shfl_xor_sync(0xffffffffu, ay, sh, kVS);
        az += __shfl_xor_sync(0xffffffffu, az, sh, kVS);
      }
      const int64_t lv = base + gidx + i * ngroups;
      if (lane == 0 && lv < nloop && wv[i] != 0.0f) {
        const int32_t v = static_cast<int32_t>(STAGED ? o.vb0 + lv : lv);
        epi(v, make_float3(ax, ay, az), wv[i]);
      }
    }
  }
}

// Init vertex phase: B_v = m_v I + sum g g^T / alpha~ and its inverse,
// rhs_v = sum (b_t / alpha~_t) g_{t,v}; r = rhs (r.w = w_v), y = yc = p = 0,
// z = B^-1 r; returns this thread's share of r.z.  One vertex per lane group
// at a time (runs once per solve).
template <bool STAGED>
__device__ __forceinline__ float vinit(const QArgs& a, const Own& o) {
  const int lane = threadIdx.x % kVS;
  int64_t gidx, ngroups, nloop;
  if (STAGED) {
    gidx = threadIdx.x / kVS;
    ngroups = blockDim.x / kVS;
    nloop = o.nvb;
  } else {
    gidx = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kVS;
    ngroups = (int64_t)gridDim.x * blockDim.x / kVS;
    nloop = a.nv;
  }
  float acc = 0.0f;
  for (int64_t base = 0; base < nloop; base += ngroups) {
    const int64_t lv = base + gidx;
    float wv = 0.0f;
    int32_t k0 = 0, k1 = 0;
    if (lv < nloop) {
      if (STAGED) {
        wv = o.w[lv];
        k0 = o.off[lv];
        k1 = o.off[lv + 1] - 1;
      } else {
        wv = a.invm[lv];
        k0 = a.inc_ptr[lv];
        k1 = a.inc_ptr[lv + 1];
      }
      if (wv == 0.0f) k1 = k0;
    }
    float h[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int32_t k = k0 + lane; k < k1; k += kVS) {
      const float4 g = STAGED ? o.e[k] : __ldg(a.gV + k);
      const int32_t t = __float_as_int(g.w);
      const float ia = 1.0f / __ldg(a.alpha + t);
      const float bt = a.b[t] * ia;
      h[0] += bt * g.x;
      h[1] += bt * g.y;
      h[2] += bt * g.z;
      h[3] += ia * g.x * g.x;
      h[4] += ia * g.x * g.y;
      h[5] += ia * g.x * g.z;
      h[6] += ia * g.y * g.y;
      h[7] += ia * g.y * g.z;
      h[8] += ia * g.z * g.z;
    }
#pragma unroll
    for (int j = 0; j < 9; ++j) {
#pragma unroll
      for (int sh = kVS / 2; sh > 0; sh >>= 1) h[j] += __shfl_xor_sync(0xffffffffu, h[j], sh, kVS);
    }
    if (lane == 0 && lv < nloop) {
      const int32_t v = static_cast<int32_t>(STAGED ? o.vb0 + lv : lv);
      float4 i0 = make_float4(0.f, 0.f, 0.f, 0.f), i1 = i0;
      float3 rv = make_float3(0.f, 0.f, 0.f);
      if (wv != 0.0f) {
        const float m = 1.0f / wv;
        const float b00 = m + h[3], b01 = h[4], b02 = h[5], b11 = m + h[6], b12 = h[7],
                    b22 = m + h[8];
        const float c00 = b11 * b22 - b12 * b12, c01 = b02 * b12 - b01 * b22,
                    c02 = b01 * b12 - b02 * b11, c11 = b00 * b22 - b02 * b02,
                    c12 = b01 * b02 - b00 * b12, c22 = b00 * b11 - b01 * b01;
        const float det = b00 * c00 + b01 * c01 + b02 * c02;
        const float id = det != 0.0f ? 1.0f / det : 0.0f;
        i0 = make_float4(c00 * id, c01 * id, c02 * id, c11 * id);
        i1 = make_float4(c12 * id, c22 * id, 0.f, 0.f);
        rv = make_float3(h[0], h[1], h[2]);
      }
      const float3 zv = binv_apply(i0, i1, rv);
      a.bi0[v] = i0;
      a.bi1[v] = i1;
      a.rhs[v] = p4(rv);
      a.r[v] = p4(rv, wv);
      a.z[v] = p4(zv);
      a.y[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.yc[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.p[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.d[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.q[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      acc += dot3(rv, zv);
    }
  }
  return acc;
}

// Largest eigenvalue of the symmetric tridiagonal (diagonal da, off-diagonal
// db) by Sturm-sequence bisection on its Gershgorin interval.
__device__ double tridiag_lmax(const double* da, const double* db, int k) {
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < k; ++i) {
    const double rr = (i > 0 ? fabs(db[i - 1]) : 0.0) + (i + 1 < k ? fabs(db[i]) : 0.0);
    lo = fmin(lo, da[i] - rr);
    hi = fmax(hi, da[i] + rr);
  }
  if (!(hi >= lo) || !isfinite(hi) || !isfinite(lo)) return NAN;
  for (int it = 0; it < 200 && hi - lo > 1e-12 * fmax(1.0, fabs(hi)); ++it) {
    const double mid = 0.5 * (lo + hi);
    int below = 0;
    double dd = 1.0;
    for (int i = 0; i < k; ++i) {
      dd = (da[i] - mid) - (i > 0 ? db[i - 1] * db[i - 1] / dd : 0.0);
      if (dd == 0.0) dd = -1e-300;
      if (dd < 0.0) ++below;
    }
    if (below >= k) hi = mid;
    else lo = mid;
  }
  return hi;
}

template <bool STAGED>
__global__ void __launch_bounds__(kPT, 1) k_pcg(QArgs a) {
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ Ctl c;
  const int G = gridDim.x;
  double* P0 = a.partials;          // p.Kp
  double* P1 = a.partials + G;      // b.b
  double* P2 = a.partials + 2 * G;  // r.z
  double* P3 = a.partials + 3 * G;  // |J W r|^2
  unsigned long long gen = 0;
  int32_t* sw = &a.st->status;

  Own o;
  if (STAGED) {
    const int32_t tb0 = a.part_t[blockIdx.x], tb1 = a.part_t[blockIdx.x + 1];
    const int32_t vb0 = a.part_v[blockIdx.x], vb1 = a.part_v[blockIdx.x + 1];
    const int32_t e0 = a.inc_ptr[vb0];
    o.tbeg = tb0 + threadIdx.x;
    o.tend = tb1;
    o.tstep = blockDim.x;
    o.vbeg = vb0 + threadIdx.x;
    o.vend = vb1;
    o.vstep = blockDim.x;
    o.tb0 = tb0;
    o.vb0 = vb0;
    o.nvb = vb1 - vb0;
    float4* se = reinterpret_cast<float4*>(s_dyn);
    int4* sq = reinterpret_cast<int4*>(se + a.emax + a.vmax);
    int32_t* soff = reinterpret_cast<int32_t*>(sq + a.tmax);
    float* sw_ = reinterpret_cast<float*>(soff + a.vmax + 1);
    // vertex lv's entries go to [off + lv, off + lv + n): one pad slot per vertex
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5, ln = threadIdx.x & 31;
    for (int lv = wid; lv < o.nvb; lv += nw) {
      const int32_t k0 = a.inc_ptr[vb0 + lv], n = a.inc_ptr[vb0 + lv + 1] - k0;
      const int32_t dst = k0 - e0 + lv;
      for (int j = ln; j < n; j += 32) se[dst + j] = __ldg(a.gV + k0 + j);
    }
    for (int k = threadIdx.x; k < tb1 - tb0; k += blockDim.x) sq[k] = a.t_i[tb0 + k];
    for (int k = threadIdx.x; k <= o.nvb; k += blockDim.x) soff[k] = a.inc_ptr[vb0 + k] - e0 + k;
    for (int k = threadIdx.x; k < o.nvb; k += blockDim.x) sw_[k] = a.invm[vb0 + k];
    o.e = se;
    o.q = sq;
    o.off = soff;
    o.w = sw_;
  } else {
    const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t T = (int64_t)G * blockDim.x;
    o.tbeg = gt;
    o.tend = a.nt;
    o.tstep = T;
    o.vbeg = gt;
    o.vend = a.nv;
    o.vstep = T;
    o.tb0 = o.vb0 = o.nvb = 0;
    o.e = nullptr;
    o.q = nullptr;
    o.off = nullptr;
    o.w = nullptr;
  }
  if (threadIdx.x == 0) {
    c.best = 1e300;
    c.amp0 = -1.0;
    c.declined = 0;
    c.since = 0;
    c.iters = 0;
    c.nboot = 0;
    c.stop = 0;
    c.status = 0;
    c.beta = 0.0;
    c.be = 0.0f;
    c.inv_theta = 1.0f;
  }
  __syncthreads();

  // B, B^-1, rhs, r, z; partials of r.z and b.b
  {
    const float rz = vinit<STAGED>(a, o);
    float bb = 0.0f;
    for (int64_t t = o.tbeg; t < o.tend; t += o.tstep) {
      const float bt = a.b[t];
      bb += bt * bt;
    }
    put_partial(rz, P2);
    put_partial(bb, P1);
  }
  if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return;
  if (threadIdx.x < 32) {
    const double sb = warp_sum_partials(P1, G);
    const double sz = warp_sum_partials(P2, G);
    if (threadIdx.x == 0) {
      c.bb = sb;
      c.rz = sz;
      const double t2 = a.tol_abs * a.tol_abs, r2 = a.tol_rel * a.tol_rel * sb;
      c.tol2 = r2 > t2 ? r2 : t2;
      if (!isfinite(sb) || !isfinite(sz)) {
        c.status |= MGPBD_STATUS_NAN;
        c.stop = 1;
      }
    }
  }
  __syncthreads();

  // PCG with preconditioner B (m = 1) or the Chebyshev polynomial in B^-1 K
  // of degree m; `boot` records the coefficients and stops after kBoot
  // iterations.  Every decision is taken by thread 0 from sums that are
  // bit-identical in all blocks.
  auto cg = [&](int m, bool boot) -> bool {
    int its = 0;
    while (!c.stop) {
      // s = J (z + beta p) / alpha~; |J W r|^2 (dual residual of y)
      {
        float e2 = 0.0f;
        tphase<kT1, STAGED>(a, o, c.be, &e2);
        put_partial(e2, P3);
      }
      if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return false;
      if (threadIdx.x < 32) {
        const double se = warp_sum_partials(P3, G);
        if (threadIdx.x == 0) {
          c.rres = se;
          if (c.amp0 < 0.0) {
            // the start y = 0, i.e. dlam = alpha~^-1 b: its dual residual
            // over |b| measures how much float32 accuracy the hand-over loses
            c.amp0 = c.bb > 0.0 ? sqrt(se / c.bb) : 0.0;
            if (a.max_amp > 0.0 && c.amp0 > a.max_amp) {
              c.declined = 1;
              c.stop = 1;
            }
          }
          if (c.stop) {
          } else if (!isfinite(se)) {
            c.status |= MGPBD_STATUS_NAN;
            c.stop = 1;
          } else if (se < c.tol2) {
            c.stop = 1;
          } else if (c.iters >= a.maxiter) {
            c.status |= MGPBD_STATUS_CG_MAXITER;
            c.stop = 1;
          } else if (a.stall_its > 0) {
            if (se < 0.81 * c.best) {
              c.best = se;
              c.since = 0;
            } else if (++c.since >= a.stall_its) {
              c.stop = 1;
            }
          }
        }
      }
      __syncthreads();
      if (c.stop || (boot && its >= kBoot)) break;
      // p = z + beta p; q = K p; partials of p.q
      {
        float pq = 0.0f;
        const float be = c.be;
        vphase<STAGED>(a, o, [&](int32_t v, float3 sum, float w) {
          const float3 zv = f3(a.z[v]), pv0 = f3(a.p[v]);
          const float3 pv = make_float3(zv.x + be * pv0.x, zv.y + be * pv0.y, zv.z + be * pv0.z);
          const float m_v = 1.0f / w;
          const float3 qv = make_float3(m_v * pv.x + sum.x, m_v * pv.y + sum.y, m_v * pv.z + sum.z);
          a.p[v] = p4(pv);
          a.q[v] = p4(qv);
          pq += dot3(pv, qv);
        });
        put_partial(pq, P0);
      }
      if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return false;
      if (threadIdx.x < 32) {
        const double sp = warp_sum_partials(P0, G);
        if (threadIdx.x == 0) {
          c.pap = sp;
          if (!isfinite(sp)) c.status |= MGPBD_STATUS_NAN;
          if (!(fabs(sp) >= 1e-30) || !isfinite(sp)) {
            c.stop = 1;
          } else {
            if (sp <= 0.0) c.status |= MGPBD_STATUS_PAP_NONPOS;
            c.alpha = c.rz / sp;
            c.al = (float)c.alpha;
            if (boot) c.ca[c.nboot] = c.alpha;
          }
        }
      }
      __syncthreads();
      if (c.stop) break;
      // y += alpha p (compensated); r -= alpha q; z = B^-1 r (m = 1) or
      // z = d = B^-1 r / theta (first Chebyshev step)
      {
        const float al = c.al, it = c.inv_theta;
        float rz = 0.0f;
        for (int64_t v = o.vbeg; v < o.vend; v += o.vstep) {
          const float4 r4 = a.r[v];
          if (r4.w == 0.0f) continue;
          const float3 pv = f3(a.p[v]), qv = f3(a.q[v]);
          float4 yv = a.y[v], cv = a.yc[v];
          {
            const float y0 = al * pv.x - cv.x, s0 = yv.x + y0;
            cv.x = (s0 - yv.x) - y0;
            yv.x = s0;
            const float y1 = al * pv.y - cv.y, s1 = yv.y + y1;
            cv.y = (s1 - yv.y) - y1;
            yv.y = s1;
            const float y2 = al * pv.z - cv.z, s2 = yv.z + y2;
            cv.z = (s2 - yv.z) - y2;
            yv.z = s2;
          }
          a.y[v] = yv;
          a.yc[v] = cv;
          const float3 rv = make_float3(r4.x - al * qv.x, r4.y - al * qv.y, r4.z - al * qv.z);
          a.r[v] = p4(rv, r4.w);
          float3 zv = binv_apply(a.bi0[v], a.bi1[v], rv);
          if (m > 1) {
            zv = make_float3(zv.x * it, zv.y * it, zv.z * it);
            a.d[v] = p4(zv);
          }
          a.z[v] = p4(zv);
          rz += dot3(rv, zv);
        }
        if (m == 1) put_partial(rz, P2);
      }
      if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return false;
      // Chebyshev steps 1..m-1: w = K z; d = c1 d + c2 B^-1 (r - w); z += d
      for (int i = 1; i < m; ++i) {
        tphase<kTZ, STAGED>(a, o, 0.0f, nullptr);
        if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return false;
        const float c1 = c.c1[i], c2 = c.c2[i];
        const bool last = i == m - 1;
        float rz = 0.0f;
        vphase<STAGED>(a, o, [&](int32_t v, float3 sum, float w) {
          const float3 zv = f3(a.z[v]), rv = f3(a.r[v]), dv = f3(a.d[v]);
          const float m_v = 1.0f / w;
          const float3 res = make_float3(rv.x - (m_v * zv.x + sum.x), rv.y - (m_v * zv.y + sum.y),
                                         rv.z - (m_v * zv.z + sum.z));
          const float3 rr = binv_apply(a.bi0[v], a.bi1[v], res);
          const float3 dn = make_float3(c1 * dv.x + c2 * rr.x, c1 * dv.y + c2 * rr.y,
                                        c1 * dv.z + c2 * rr.z);
          const float3 zn = make_float3(zv.x + dn.x, zv.y + dn.y, zv.z + dn.z);
          a.d[v] = p4(dn);
          a.z[v] = p4(zn);
          if (last) rz += dot3(rv, zn);
        });
        if (last) put_partial(rz, P2);
        if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return false;
      }
      if (threadIdx.x < 32) {
        const double sz = warp_sum_partials(P2, G);
        if (threadIdx.x == 0) {
          c.iters += 1;
          if (!isfinite(sz)) {
            c.status |= MGPBD_STATUS_NAN;
            c.stop = 1;
          } else if (fabs(c.rz) < 1e-30) {
            c.stop = 1;
          } else {
            c.beta = sz / c.rz;
            c.rz = sz;
            c.be = (float)c.beta;
            if (boot) {
              c.cb[c.nboot] = c.beta;
              c.nboot += 1;
            }
          }
        }
      }
      __syncthreads();
      ++its;
    }
    return true;
  };

  const int m = a.degree;
  if (!cg(1, m > 1)) return;
  if (m > 1 && !c.stop) {
    // lambda_max of B^-1 K from the bootstrap's Lanczos tridiagonal, the
    // Chebyshev coefficients, and a restart from the current y
    if (threadIdx.x == 0) {
      const int n = c.nboot;
      double da[kBoot], db[kBoot];
      for (int j = 0; j < n; ++j) {
        da[j] = 1.0 / c.ca[j] + (j > 0 ? c.cb[j - 1] / c.ca[j - 1] : 0.0);
        db[j] = sqrt(fmax(c.cb[j], 0.0)) / c.ca[j];
      }
      double lmax = n > 0 ? tridiag_lmax(da, db, n) : NAN;
      if (!isfinite(lmax) || !(lmax > 0.0)) {
        c.status |= MGPBD_STATUS_NAN;
        lmax = 2.0;
      }
      const double hi = 1.02 * lmax, lo = hi * a.cheb_lo;
      const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
      double rho = 1.0 / sigma;
      for (int i = 1; i < m; ++i) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        c.c1[i] = (float)(rn * rho);
        c.c2[i] = (float)(2.0 * rn / delta);
        rho = rn;
      }
      c.inv_theta = (float)(1.0 / theta);
      c.beta = 0.0;
      c.be = 0.0f;
    }
    __syncthreads();
    // r = rhs - K y; z = d = B^-1 r / theta
    tphase<kTY, STAGED>(a, o, 0.0f, nullptr);
    if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return;
    {
      const float it = c.inv_theta;
      vphase<STAGED>(a, o, [&](int32_t v, float3 sum, float w) {
        const float3 yv = f3(a.y[v]), hv = f3(a.rhs[v]);
        const float m_v = 1.0f / w;
        const float3 rv = make_float3(hv.x - (m_v * yv.x + sum.x), hv.y - (m_v * yv.y + sum.y),
                                      hv.z - (m_v * yv.z + sum.z));
        float3 zv = binv_apply(a.bi0[v], a.bi1[v], rv);
        zv = make_float3(zv.x * it, zv.y * it, zv.z * it);
        a.r[v] = p4(rv, w);
        a.z[v] = p4(zv);
        a.d[v] = p4(zv);
      });
    }
    if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return;
    for (int i = 1; i < m; ++i) {
      tphase<kTZ, STAGED>(a, o, 0.0f, nullptr);
      if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return;
      const float c1 = c.c1[i], c2 = c.c2[i];
      const bool last = i == m - 1;
      float rz = 0.0f;
      vphase<STAGED>(a, o, [&](int32_t v, float3 sum, float w) {
        const float3 zv = f3(a.z[v]), rv = f3(a.r[v]), dv = f3(a.d[v]);
        const float m_v = 1.0f / w;
        const float3 res = make_float3(rv.x - (m_v * zv.x + sum.x), rv.y - (m_v * zv.y + sum.y),
                                       rv.z - (m_v * zv.z + sum.z));
        const float3 rr = binv_apply(a.bi0[v], a.bi1[v], res);
        const float3 dn =
            make_float3(c1 * dv.x + c2 * rr.x, c1 * dv.y + c2 * rr.y, c1 * dv.z + c2 * rr.z);
        const float3 zn = make_float3(zv.x + dn.x, zv.y + dn.y, zv.z + dn.z);
        a.d[v] = p4(dn);
        a.z[v] = p4(zn);
        if (last) rz += dot3(rv, zn);
      });
      if (last) put_partial(rz, P2);
      if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return;
    }
    if (threadIdx.x < 32) {
      const double sz = warp_sum_partials(P2, G);
      if (threadIdx.x == 0) {
        c.rz = sz;
        if (!isfinite(sz)) {
          c.status |= MGPBD_STATUS_NAN;
          c.stop = 1;
        }
      }
    }
    __syncthreads();
    if (!cg(m, false)) return;
  }

  // y -= yc (the compensated sum), then dlam = (b - J y) / alpha~
  for (int64_t v = o.vbeg; v < o.vend; v += o.vstep) {
    const float4 yv = a.y[v], cv = a.yc[v];
    a.y[v] = make_float4(yv.x - cv.x, yv.y - cv.y, yv.z - cv.z, 0.0f);
  }
  if (!grid_sync(a.gs, sw, a.spin_ns, gen)) return;
  tphase<kTFinal, STAGED>(a, o, 0.0f, nullptr);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    CgState* st = a.st;
    st->rz = c.rz;
    st->pap = c.pap;
    st->alpha = c.alpha;
    st->beta = c.beta;
    st->rr = c.rres;
    st->rr0 = c.bb;
    st->tol2 = c.tol2;
    st->iters = c.iters;
    st->done = 1;
    st->maxiter = a.maxiter;
    st->body_runs = c.nboot;
    st->flags = c.declined;
    st->rz_new = c.amp0;
    atomicOr(reinterpret_cast<unsigned int*>(&st->status), c.status);
  }
}

int64_t staged_smem_bytes(int32_t emax, int32_t tmax, int32_t vmax) {
  const int64_t b = 16LL * (emax + vmax) + 16LL * tmax + 4LL * (vmax + 1) + 4LL * vmax;
  return (b + 15) / 16 * 16;
}

}  // namespace

bool pcg_plan_fits(JcgPlan& plan) {
  if (!plan.staged) return true;
  const int64_t smem = staged_smem_bytes(plan.emax, plan.tmax, plan.vmax);
  int dev = 0, optin = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem > optin) return false;
  MGPBD_CUDA(cudaFuncSetAttribute(k_pcg<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
  int occ = 0;
  MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pcg<true>, kPT,
                                                           static_cast<size_t>(smem)));
  return occ >= 1;
}

int pcg_unstaged_grid() {
  int dev = 0, sms = 0, occ = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pcg<false>, kPT, 0));
  require(occ >= 1, MGPBD_ENOTSUP, "primal CG kernel does not fit on an SM");
  return sms * occ;
}

void launch_pcg_primal(const JView& j, const PcgVecs& v, const JcgPlan& plan,
                       const int32_t* part_dev, CgState* st, double tol_abs, double tol_rel,
                       int maxiter, int degree, float cheb_lo, int stall_its, double max_amp,
                       double spin_limit_s, cudaStream_t s) {
  require(degree >= 1 && degree <= kMaxCheb, MGPBD_EINVAL, "Chebyshev degree out of range");
  require(plan.grid > 0, MGPBD_ESTATE, "persistent CG plan not built");
  require(4LL * plan.grid <= v.partials_capacity, MGPBD_ERANGE, "partials buffer too small");
  require(!plan.staged || part_dev != nullptr, MGPBD_ESTATE, "staged plan without partition");
  QArgs a;
  a.nt = j.nt;
  a.nv = j.nv;
  a.n4 = j.n4;
  a.gE = j.gE;
  a.qE = j.qE;
  require(j.n4 >= j.nt || (j.gE && j.qE), MGPBD_ESTATE, "compact length constraints not prepared");
  a.t_i = reinterpret_cast<const int4*>(j.t_i);
  require(j.gT != nullptr, MGPBD_ESTATE, "persistent CG needs the gradient planes");
  a.gradC = j.gT;
  a.alpha = j.alpha;
  a.invm = j.invm;
  a.inc_ptr = j.inc_ptr;
  a.gV = j.gV;
  a.b = v.b;
  a.dlam = v.dlam;
  a.y = v.y;
  a.yc = v.yc;
  a.r = v.r;
  a.z = v.z;
  a.d = v.d;
  a.p = v.p;
  a.q = v.q;
  a.rhs = v.rhs;
  a.bi0 = v.bi0;
  a.bi1 = v.bi1;
  a.s = v.s;
  a.partials = v.partials;
  a.gs = v.gs;
  a.st = st;
  a.part_v = plan.staged ? part_dev : nullptr;
  a.part_t = plan.staged ? part_dev + plan.grid + 1 : nullptr;
  a.emax = plan.emax;
  a.tmax = plan.tmax;
  a.vmax = plan.vmax;
  a.tol_abs = tol_abs;
  a.tol_rel = tol_rel;
  a.maxiter = maxiter;
  a.degree = degree;
  a.cheb_lo = cheb_lo;
  a.stall_its = stall_its;
  a.max_amp = max_amp;
  a.spin_ns = static_cast<unsigned long long>(spin_limit_s * 1e9);
  MGPBD_CUDA(cudaMemsetAsync(v.gs, 0, sizeof(GridSync), s));
  MGPBD_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), s));
  void* args[] = {&a};
  const void* fn = plan.staged ? reinterpret_cast<const void*>(k_pcg<true>)
                               : reinterpret_cast<const void*>(k_pcg<false>);
  const size_t smem = plan.staged ? static_cast<size_t>(staged_smem_bytes(plan.emax, plan.tmax,
                                                                           plan.vmax))
                                  : 0;
  // per-function attribute shared by every handle: set this plan's limit
  if (plan.staged)
    MGPBD_CUDA(cudaFuncSetAttribute(k_pcg<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
  MGPBD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(plan.grid), dim3(kPT), args, smem, s));
  MGPBD_CHECK_LAUNCH();
}

}  // namespace mgpbd
