// The Chebyshev-preconditioned CG of FAST mode as ONE cooperative
// persistent kernel per solve.
//
// Every phase of an iteration (vertex phase, tet phase, vector update) runs
// on all blocks of one resident grid, separated by a grid barrier, instead
// of one kernel launch per phase: a launch costs each SM ~3 us of ramp-up
// and drain around ~4 us of work here, and a degree-k iteration has 2k + 1
// phases.  Scalars (alpha, beta, the stopping test) never leave the chip:
// each block writes its partial of a dot product, and after the barrier
// warp 0 of every block sums all partials in the same fixed order, so all
// blocks hold bit-identical scalars and take the same branch.
//
// Staging: when the mesh is small enough (up to ~400k tets on 152 SMs),
// each block owns a contiguous range of vertices (balanced by incident
// entries plus a per-vertex weight) and of tets (32-aligned), and copies
// their constant operator data into shared memory once per solve: the
// vertex-major entries (gradient, tet id), the incidence offsets and
// weights, and the tet indices.  A phase then issues only the gathers of the vector it applies
// A to (x_t in the vertex phase, u_v in the tet phase) plus the coalesced
// per-tet loads, instead of two or three dependent L2 round trips.
// Larger meshes run the same phases reading everything from L2, with tets
// and vertices strided over the grid.
//
// Arithmetic is float32 per element (GB300's float64 rate is a small
// fraction of its float32 rate).  Dot products sum in float32 within a warp
// and in float64 across warps and blocks; the solution is accumulated with
// Kahan compensation (Kahan 1965) so ~10^3 updates do not lose its low bits.
//
// Barrier waits are bounded: a block that waits longer than the given limit
// marks the solve failed (status bit, error flag) and returns, and every
// other block leaves at its next wait; the host reports the failure.
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

// Staged: one block of kPT threads per SM, up to 112 registers a thread,
// so each thread can issue the gathers of several tets (vertices) before
// it uses them, and 152 arrivals per grid barrier.  Unstaged: two blocks
// per SM (56 registers a thread): the phases wait on L2 gathers, and twice
// the resident warps hide more of that latency than the extra registers
// would.
constexpr int kPT = 576;
constexpr int kTB = 4;   // tets a thread handles per round of a tet phase
constexpr int kVS = 4;   // lanes per vertex in the staged vertex phase
constexpr int kVE = 6;   // entries a lane gathers per vertex and round
constexpr int kVB = 4;   // vertices a lane group handles per round
constexpr int kVertexCost = 64;  // per-vertex weight of the work split

struct PArgs {
  TArgs ta;  // t_i, gradC, u, alpha~, 1/diag, nt
  int32_t nv;
  const int32_t* inc_ptr;
  const float4* gV;
  const float* invm;
  float4* u;
  const float* b;
  float* x;
  float* xc;
  float* r;
  float* z;
  float* d;
  float* p;
  float* ap;
  double* partials;  // 3 slots of gridDim.x
  GridSync* gs;
  CgState* st;
  const JState* js;
  const int32_t* part_v;  // staged: block vertex ranges (grid + 1)
  const int32_t* part_t;  // staged: block tet ranges (grid + 1)
  int32_t emax, tmax, vmax;
  double tol_abs, tol_rel;
  int32_t maxiter, degree;
  int32_t warm;  // 1: start from the x on entry instead of 0
  float4* ulo;   // warm start: low part of u (u = a.u + ulo, float64 sums)
  unsigned long long spin_ns;
  int32_t unit_dinv;  // 1: 1/diag is all ones (unscaled base): skip its loads
  const JcgCtl* ctl;  // device-side tolerance / limit / start, or null
};

// (the staged kernel keeps the loads: the flag's test spills a register
// there, and its operator sits in shared memory anyway)
template <bool STAGED>
__device__ __forceinline__ float dinv_of(const PArgs& a, int64_t t) {
  return (!STAGED && a.unit_dinv) ? 1.0f : __ldg(a.ta.dinv + t);
}

// This block's share of the work: tets from tbeg to tend in steps of tstep
// (staged: the block's own range; otherwise strided over the whole grid),
// and, when staged, its vertex range and the shared-memory copies.
struct Own {
  int64_t tbeg, tend, tstep;
  int32_t tb0;
  int32_t vb0, nvb;
  const float4* e;     // entries of the block's vertices
  const int4* q;       // indices of the block's tets
  const int32_t* off;  // nvb + 1 entry offsets
  const float* w;      // nvb vertex weights
};

__device__ __forceinline__ bool grid_sync(const PArgs& a, unsigned long long& gen) {
  return pdev::grid_sync(a.gs, &a.st->status, a.spin_ns, gen);
}

// sum_l g_{t,l} . u_{q_l} for tet t with indices q (a.gradC: the three
// gradient planes)
__device__ __forceinline__ float tdot(const TArgs& a, int64_t t, int4 q) {
  const float4 g0 = __ldg(a.gradC + t), g1 = __ldg(a.gradC + a.nt + t),
               g2 = __ldg(a.gradC + 2LL * a.nt + t);
  const float4 u0 = a.u[q.x], u1 = a.u[q.y], u2 = a.u[q.z], u3 = a.u[q.w];
  return (g0.x * u0.x + g0.y * u0.y + g0.z * u0.z) + (g0.w * u1.x + g1.x * u1.y + g1.y * u1.z) +
         (g1.z * u2.x + g1.w * u2.y + g2.x * u2.z) + (g2.y * u3.x + g2.z * u3.y + g2.w * u3.z);
}

// A t of constraint t: staged blocks use their shared copy of the indices;
// unstaged, length constraints (t >= n4) take the compact two-vertex path
template <bool STAGED>
__device__ __forceinline__ float tdot_any(const PArgs& a, const Own& o, int64_t t);

template <bool STAGED>
__device__ __forceinline__ int4 tet_q(const PArgs& a, const Own& o, int64_t t) {
  if (STAGED) return o.q[t - o.tb0];
  return a.ta.t_i[t];
}

template <bool STAGED>
__device__ __forceinline__ float tdot_any(const PArgs& a, const Own& o, int64_t t) {
  if (!STAGED && t >= a.ta.n4) return jt_edge(a.ta, t);
  return tdot(a.ta, t, tet_q<STAGED>(a, o, t));
}

// Warm start, vertex phase in float64: u_v = w_v sum x_t g_{t,l} summed in
// float64 and stored as a float pair (a.u = rounded sum, a.ulo = the rest).
// The residual b - A x of a good start x is a small difference of large
// terms; float32 sums would bury it in their rounding (~1e-7 of the terms),
// and CG would then converge to the wrong target.  Runs once per solve.
template <bool STAGED>
__device__ __forceinline__ void vphase_warm(const PArgs& a, const Own& o) {
  const int lane = threadIdx.x % 4;
  int64_t gidx, ngroups, nloop;
  if (STAGED) {
    gidx = threadIdx.x / 4;
    ngroups = blockDim.x / 4;
    nloop = o.nvb;
  } else {
    gidx = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 4;
    ngroups = (int64_t)gridDim.x * blockDim.x / 4;
    nloop = a.nv;
  }
  for (int64_t base = 0; base < nloop; base += ngroups) {
    const int64_t lv = base + gidx;
    float w = 0.0f;
    int32_t k0 = 0, k1 = 0;
    if (lv < nloop) {
      if (STAGED) {
        w = o.w[lv];
        k0 = o.off[lv];
        k1 = o.off[lv + 1] - 1;
      } else {
        w = a.invm[lv];
        k0 = a.inc_ptr[lv];
        k1 = a.inc_ptr[lv + 1];
      }
    }
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int32_t k = k0 + lane; k < k1; k += 4) {
      const float4 g = STAGED ? o.e[k] : __ldg(a.gV + k);
      const double xt = a.x[__float_as_int(g.w)];
      sx += xt * g.x;
      sy += xt * g.y;
      sz += xt * g.z;
    }
#pragma unroll
    for (int sh = 2; sh > 0; sh >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, sh, 4);
      sy += __shfl_xor_sync(0xffffffffu, sy, sh, 4);
      sz += __shfl_xor_sync(0xffffffffu, sz, sh, 4);
    }
    if (lane == 0 && lv < nloop) {
      const int64_t v = STAGED ? o.vb0 + lv : lv;
      sx *= w;
      sy *= w;
      sz *= w;
      const float hx = (float)sx, hy = (float)sy, hz = (float)sz;
      a.u[v] = make_float4(hx, hy, hz, 0.0f);
      a.ulo[v] = make_float4((float)(sx - hx), (float)(sy - hy), (float)(sz - hz), 0.0f);
    }
  }
}

// (A x)_t in float64 from the float pair u + ulo (warm start)
template <bool STAGED>
__device__ __forceinline__ double tdot_warm(const PArgs& a, const Own& o, int64_t t) {
  const int4 q = tet_q<STAGED>(a, o, t);
  const int32_t vs[4] = {q.x, q.y, q.z, q.w};
  const float4 g0 = __ldg(a.ta.gradC + t), g1 = __ldg(a.ta.gradC + a.ta.nt + t),
               g2 = __ldg(a.ta.gradC + 2LL * a.ta.nt + t);
  const float gg[12] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w, g2.x, g2.y, g2.z, g2.w};
  double acc = 0.0;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const float4 hi = a.u[vs[l]], lo = a.ulo[vs[l]];
    acc += (double)gg[3 * l] * ((double)hi.x + lo.x) + (double)gg[3 * l + 1] * ((double)hi.y + lo.y) +
           (double)gg[3 * l + 2] * ((double)hi.z + lo.z);
  }
  return acc + (double)__ldg(a.ta.alpha + t) * a.x[t];
}

// Vertex phase: u_v = w_v sum x_t g_{t,l} with x_t = src_t (+ beta p_t).
template <int SRC, bool STAGED>
__device__ __forceinline__ void vphase(const PArgs& a, const Own& o, float beta, const float* src) {
  if (!STAGED) {
    const int lane = threadIdx.x % kVG;
    constexpr int kPerWarp = 32 / kVG;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t stride = ((int64_t)gridDim.x * blockDim.x >> 5) * kPerWarp;
    for (int64_t base = warp * kPerWarp; base < a.nv; base += stride) {
      const int64_t v = base + (threadIdx.x & 31) / kVG;
      const bool valid = v < a.nv;
      float w;
      const float3 s = jv_group<SRC>(v, valid, lane, a.inc_ptr, a.gV, a.invm, src, a.p, beta, &w);
      if (valid && lane == 0) a.u[v] = make_float4(w * s.x, w * s.y, w * s.z, 0.0f);
    }
    return;
  }
  // staged: kVS lanes per vertex, kVB vertices per lane group and round;
  // the entries (shared memory, one pad slot after each vertex's run so
  // consecutive vertices start 4 banks apart) give the tet ids, and all
  // gathers of a round are issued before any is consumed
  const int lane = threadIdx.x % kVS;
  const int grp = threadIdx.x / kVS;
  const int ngrp = blockDim.x / kVS;
  for (int base = 0; base < o.nvb; base += kVB * ngrp) {
    int k0[kVB], k1[kVB];
    float wv[kVB];
#pragma unroll
    for (int i = 0; i < kVB; ++i) {
      const int lv = base + grp + i * ngrp;
      k0[i] = k1[i] = 0;
      wv[i] = 0.0f;
      if (lv < o.nvb) {
        wv[i] = o.w[lv];
        if (wv[i] != 0.0f) {
          k0[i] = o.off[lv];
          k1[i] = o.off[lv + 1] - 1;
        }
      }
    }
    float xs[kVB][kVE];
#pragma unroll
    for (int i = 0; i < kVB; ++i) {
#pragma unroll
      for (int c = 0; c < kVE; ++c) {
        const int k = k0[i] + lane + kVS * c;
        float xt = 0.0f;
        if (k < k1[i]) {
          const int32_t t = __float_as_int(o.e[k].w);
          xt = SRC == kSrcZbP ? src[t] + beta * a.p[t] : src[t];
        }
        xs[i][c] = xt;
      }
    }
#pragma unroll
    for (int i = 0; i < kVB; ++i) {
      float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
      for (int c = 0; c < kVE; ++c) {
        const int k = k0[i] + lane + kVS * c;
        if (k < k1[i]) {
          const float4 g = o.e[k];
          ax += xs[i][c] * g.x;
          ay += xs[i][c] * g.y;
          az += xs[i][c] * g.z;
        }
      }
      // vertices with more than kVS * kVE incident tets
      for (int k = k0[i] + lane + kVS * kVE; k < k1[i]; k += kVS) {
        const float4 g = o.e[k];
        const int32_t t = __float_as_int(g.w);
        const float xt = SRC == kSrcZbP ? src[t] + beta * a.p[t] : src[t];
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
      const int lv = base + grp + i * ngrp;
      if (lane == 0 && lv < o.nvb)
        a.u[o.vb0 + lv] = make_float4(wv[i] * ax, wv[i] * ay, wv[i] * az, 0.0f);
    }
  }
}

// Chebyshev step: rr = D^-1 (r - A z); d = c1 d + c2 rr; z += d.  LAST also
// writes this block's partial of r.z.
template <bool LAST, bool STAGED>
__device__ __forceinline__ void tphase_cheb(const PArgs& a, const Own& o, float c1, float c2,
                                            double* slot) {
  float acc = 0.0f;
  for (int64_t tb = o.tbeg; tb < o.tend; tb += kTB * o.tstep) {
    float y[kTB];
#pragma unroll
    for (int i = 0; i < kTB; ++i) {
      const int64_t t = tb + i * o.tstep;
      y[i] = t < o.tend ? tdot_any<STAGED>(a, o, t) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < kTB; ++i) {
      const int64_t t = tb + i * o.tstep;
      if (t < o.tend) {
        const float zt = a.z[t];
        const float yt = y[i] + __ldg(a.ta.alpha + t) * zt;
        const float rt = a.r[t];
        const float rrv = dinv_of<STAGED>(a, t) * (rt - yt);
        const float dt = c1 * a.d[t] + c2 * rrv;
        a.d[t] = dt;
        const float zn = zt + dt;
        a.z[t] = zn;
        if (LAST) acc += rt * zn;
      }
    }
  }
  if (LAST) put_partial(acc, slot);
}

// p = z + beta p; ap = A p; this block's partial of p.Ap
template <bool STAGED>
__device__ __forceinline__ void tphase_ap(const PArgs& a, const Own& o, float bf, double* slot) {
  float acc = 0.0f;
  for (int64_t tb = o.tbeg; tb < o.tend; tb += kTB * o.tstep) {
    float y[kTB];
#pragma unroll
    for (int i = 0; i < kTB; ++i) {
      const int64_t t = tb + i * o.tstep;
      y[i] = t < o.tend ? tdot_any<STAGED>(a, o, t) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < kTB; ++i) {
      const int64_t t = tb + i * o.tstep;
      if (t < o.tend) {
        const float pt = a.z[t] + bf * a.p[t];
        const float yt = y[i] + __ldg(a.ta.alpha + t) * pt;
        a.p[t] = pt;
        a.ap[t] = yt;
        acc += pt * yt;
      }
    }
  }
  put_partial(acc, slot);
}

template <bool STAGED>
__global__ void __launch_bounds__(kPT, STAGED ? 1 : 2) k_jcg(PArgs a) {
  // a skipped launch leaves before its first barrier in every block (every
  // thread reads the same flag)
  if (a.ctl && a.ctl->skip) return;
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ float s_c1[kMaxCheb], s_c2[kMaxCheb];
  __shared__ float s_scal;  // alpha or beta, broadcast from thread 0
  __shared__ int s_stop;
  // CG scalars, read and written by thread 0 only (shared memory keeps them
  // out of every thread's registers)
  __shared__ double bbs, tol2, rz, rr, pap, alpha, beta;
  __shared__ int32_t iters;
  __shared__ uint32_t status;
  if (threadIdx.x < kMaxCheb) {
    s_c1[threadIdx.x] = a.js->cf.c1[threadIdx.x];
    s_c2[threadIdx.x] = a.js->cf.c2[threadIdx.x];
  }
  // the control values, in shared memory (kept out of the registers of the
  // iteration loop): from ctl when given, else the launch arguments
  __shared__ int32_t warm, maxiter;
  __shared__ double tol_abs;
  if (threadIdx.x == 0) {
    bbs = tol2 = rz = rr = pap = alpha = beta = 0.0;
    iters = 0;
    status = 0;
    warm = a.ctl ? a.ctl->warm : a.warm;
    maxiter = a.ctl ? a.ctl->maxiter : a.maxiter;
    tol_abs = a.ctl ? a.ctl->tol_abs : a.tol_abs;
  }
  const float it = a.js->cf.inv_theta;
  const int m = a.degree;
  const int G = gridDim.x;
  double* P0 = a.partials;
  double* P1 = a.partials + G;
  double* P2 = a.partials + 2 * G;
  unsigned long long gen = 0;

  Own o;
  if (STAGED) {
    const int32_t tb0 = a.part_t[blockIdx.x], tb1 = a.part_t[blockIdx.x + 1];
    const int32_t vb0 = a.part_v[blockIdx.x], vb1 = a.part_v[blockIdx.x + 1];
    const int32_t e0 = a.inc_ptr[vb0], ne = a.inc_ptr[vb1] - e0;
    o.tbeg = tb0 + threadIdx.x;
    o.tend = tb1;
    o.tstep = blockDim.x;
    o.tb0 = tb0;
    o.vb0 = vb0;
    o.nvb = vb1 - vb0;
    float4* se = reinterpret_cast<float4*>(s_dyn);
    int4* sq = reinterpret_cast<int4*>(se + a.emax + a.vmax);
    int32_t* soff = reinterpret_cast<int32_t*>(sq + a.tmax);
    float* sw = reinterpret_cast<float*>(soff + a.vmax + 1);
    // vertex lv's entries go to [off + lv, off + lv + n): one pad slot per vertex
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5, ln = threadIdx.x & 31;
    for (int lv = wid; lv < o.nvb; lv += nw) {
      const int32_t k0 = a.inc_ptr[vb0 + lv], n = a.inc_ptr[vb0 + lv + 1] - k0;
      const int32_t dst = k0 - e0 + lv;
      for (int j = ln; j < n; j += 32) se[dst + j] = __ldg(a.gV + k0 + j);
    }
    for (int k = threadIdx.x; k < tb1 - tb0; k += blockDim.x) sq[k] = a.ta.t_i[tb0 + k];
    for (int k = threadIdx.x; k <= o.nvb; k += blockDim.x) soff[k] = a.inc_ptr[vb0 + k] - e0 + k;
    for (int k = threadIdx.x; k < o.nvb; k += blockDim.x) sw[k] = a.invm[vb0 + k];
    (void)ne;
    o.e = se;
    o.q = sq;
    o.off = soff;
    o.w = sw;
  } else {
    o.tbeg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    o.tend = a.ta.nt;
    o.tstep = (int64_t)G * blockDim.x;
    o.tb0 = 0;
    o.vb0 = 0;
    o.nvb = 0;
    o.e = nullptr;
    o.q = nullptr;
    o.off = nullptr;
    o.w = nullptr;
  }
  __syncthreads();

  // x = 0 (or the warm start x0), r = b - A x, p = 0, z = d = D^-1 r / theta;
  // partials of b.b and r.z
  if (warm) {
    vphase_warm<STAGED>(a, o);
    if (!grid_sync(a, gen)) return;
  }
  {
    float bb = 0.0f, bz = 0.0f, br = 0.0f;
    for (int64_t t = o.tbeg; t < o.tend; t += o.tstep) {
      const float bt = a.b[t];
      float rt = bt;
      if (warm) {
        rt = (float)((double)bt - tdot_warm<STAGED>(a, o, t));
      } else {
        a.x[t] = 0.0f;
      }
      a.xc[t] = 0.0f;
      a.r[t] = rt;
      a.p[t] = 0.0f;
      const float zt = dinv_of<STAGED>(a, t) * rt * it;
      a.z[t] = zt;
      a.d[t] = zt;
      bb += bt * bt;
      bz += rt * zt;
      br += rt * rt;
    }
    put_partial(bb, P0);
    put_partial(bz, P1);
    // a warm start may already meet the tolerance (a float64 residual
    // replacement after a converged solve): its r.r decides below; P2 is
    // first rewritten after the next grid barrier
    if (warm) put_partial(br, P2);
  }
  if (!grid_sync(a, gen)) return;
  if (threadIdx.x < 32) {
    const double sb = warp_sum_partials(P0, G);
    const double sz = warp_sum_partials(P1, G);
    const double s0 = warm ? warp_sum_partials(P2, G) : sb;
    if (threadIdx.x == 0) {
      bbs = sb;
      rz = sz;
      rr = s0;
      const double t2 = tol_abs * tol_abs, r2 = a.tol_rel * a.tol_rel * bbs;
      tol2 = r2 > t2 ? r2 : t2;
      int stop = maxiter <= 0 || (warm && rr < tol2);
      if (!isfinite(bbs)) {
        status |= MGPBD_STATUS_NAN;
        stop = 1;
      }
      s_stop = stop;
    }
  }
  __syncthreads();
  bool done = s_stop != 0;

  // remaining Chebyshev steps of z = M^-1 r
  if (!done && m > 1) {
    for (int i = 1; i < m; ++i) {
      vphase<kSrcX, STAGED>(a, o, 0.0f, a.z);
      if (!grid_sync(a, gen)) return;
      if (i == m - 1) tphase_cheb<true, STAGED>(a, o, s_c1[i], s_c2[i], P2);
      else tphase_cheb<false, STAGED>(a, o, s_c1[i], s_c2[i], P2);
      if (!grid_sync(a, gen)) return;
    }
    if (threadIdx.x < 32) {
      const double sz = warp_sum_partials(P2, G);
      if (threadIdx.x == 0) {
        rz = sz;
        int stop = 0;
        if (!isfinite(rz)) {
          status |= MGPBD_STATUS_NAN;
          stop = 1;
        }
        s_stop = stop;
      }
    }
    __syncthreads();
    done = s_stop != 0;
  }

  float bf = 0.0f;  // beta
  while (!done) {
    // u = W J^T (z + beta p)
    vphase<kSrcZbP, STAGED>(a, o, bf, a.z);
    if (!grid_sync(a, gen)) return;
    // p = z + beta p; ap = A p; partials of p.Ap
    tphase_ap<STAGED>(a, o, bf, P0);
    if (!grid_sync(a, gen)) return;
    if (threadIdx.x < 32) {
      const double sp = warp_sum_partials(P0, G);
      if (threadIdx.x == 0) {
        pap = sp;
        int stop = 0;
        if (!isfinite(pap)) status |= MGPBD_STATUS_NAN;
        if (!(fabs(pap) >= 1e-30) || !isfinite(pap)) {
          stop = 1;
        } else {
          if (pap <= 0.0) status |= MGPBD_STATUS_PAP_NONPOS;
          alpha = rz / pap;
          s_scal = (float)alpha;
        }
        s_stop = stop;
      }
    }
    __syncthreads();
    if (s_stop) break;
    // x += alpha p (compensated); r -= alpha Ap; z = d = D^-1 r / theta;
    // partials of r.r and r.z
    {
      const float al = s_scal;
      float acc_rr = 0.0f, acc_rz = 0.0f;
      for (int64_t t = o.tbeg; t < o.tend; t += o.tstep) {
        const float pt = a.p[t], apt = a.ap[t];
        const float s = a.x[t];
        const float y = al * pt - a.xc[t];
        const float sn = s + y;
        a.xc[t] = (sn - s) - y;
        a.x[t] = sn;
        const float rt = a.r[t] - al * apt;
        a.r[t] = rt;
        const float zt = dinv_of<STAGED>(a, t) * rt * it;
        a.z[t] = zt;
        a.d[t] = zt;
        acc_rr += rt * rt;
        acc_rz += rt * zt;
      }
      put_partial(acc_rr, P1);
      if (m == 1) put_partial(acc_rz, P2);
    }
    if (!grid_sync(a, gen)) return;
    if (threadIdx.x < 32) {
      const double sr = warp_sum_partials(P1, G);
      if (threadIdx.x == 0) {
        rr = sr;
        int stop = 0;
        if (!isfinite(rr)) {
          status |= MGPBD_STATUS_NAN;
          stop = 1;
        } else if (rr < tol2) {
          iters += 1;
          stop = 1;
        }
        s_stop = stop;
      }
    }
    __syncthreads();
    if (s_stop) break;
    if (m > 1) {
      for (int i = 1; i < m; ++i) {
        vphase<kSrcX, STAGED>(a, o, 0.0f, a.z);
        if (!grid_sync(a, gen)) return;
        if (i == m - 1) tphase_cheb<true, STAGED>(a, o, s_c1[i], s_c2[i], P2);
        else tphase_cheb<false, STAGED>(a, o, s_c1[i], s_c2[i], P2);
        if (!grid_sync(a, gen)) return;
      }
    }
    if (threadIdx.x < 32) {
      const double sz = warp_sum_partials(P2, G);
      if (threadIdx.x == 0) {
        iters += 1;
        int stop = 0;
        if (fabs(rz) < 1e-30) {
          stop = 1;
        } else {
          beta = sz / rz;
          rz = sz;
          s_scal = (float)beta;
          if (iters >= maxiter) {
            status |= MGPBD_STATUS_CG_MAXITER;
            stop = 1;
          }
        }
        s_stop = stop;
      }
    }
    __syncthreads();
    if (s_stop) break;
    bf = s_scal;
  }

  // the compensated sum, rounded once; xc keeps what the rounding dropped
  // (x + xc is the solution as a float pair, for the float64 scatter)
  for (int64_t t = o.tbeg; t < o.tend; t += o.tstep) {
    const float s = a.x[t], c = a.xc[t];
    const float hi = s - c;
    a.xc[t] = (s - hi) - c;
    a.x[t] = hi;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    CgState* st = a.st;
    st->rz = rz;
    st->pap = pap;
    st->alpha = alpha;
    st->beta = beta;
    st->rr = rr;
    st->rr0 = bbs;
    st->tol2 = tol2;
    st->iters = iters;
    st->done = 1;
    st->maxiter = maxiter;
    st->body_runs = 1;
    atomicOr(reinterpret_cast<unsigned int*>(&st->status), status);
  }
}

// ---------------------------------------------------------------------------
// Per-body CG of packed bodies (block-diagonal A): one CG per body, run in
// lockstep inside one persistent launch.  Every dot product is summed per
// body (chunks of at most kCgChunk constraints, each inside one body, one
// warp per chunk; then one warp per body over its chunks, in order), and
// alpha, beta and the stopping test are the body's own, so a stiff body no
// longer holds the others to its iteration count, nor they it to theirs:
// each converges as its own CG would.  A body that meets its bound keeps
// its x and r (its chunks are skipped); the launch ends when every body has
// stopped.  The Chebyshev preconditioner (one polynomial) and the vertex
// and tet phases are those of k_jcg, unstaged.
//
// Per iteration: vertex phase, A p (chunked), body alphas, update
// (chunked), body residuals, the Chebyshev steps (the last chunked), body
// betas: 2k + 4 barriers for degree k.

// chunk c of the per-warp loop: its constraint range and body
__device__ __forceinline__ int64_t gwarp() {
  return (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ int64_t nwarps() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }

// sum over body k's chunks (ascending) of plane q of the chunk partials;
// all lanes of the warp get it
__device__ __forceinline__ double body_total(const BodyCg& b, int q, int32_t k) {
  const int lane = threadIdx.x & 31;
  const double* cp = b.cp + (int64_t)q * b.nch;
  double acc = 0.0;
  for (int32_t i = b.bptr[k] + lane; i < b.bptr[k + 1]; i += 32) acc += __ldcg(cp + b.bidx[i]);
  return warp_sum_d(acc);
}

// Vertex phase with a per-body beta: u_v = w_v sum (z_t + beta_b(t) p_t) g_{t,l}
__device__ __forceinline__ void vphase_body_zbp(const PArgs& a, const BodyCg& b) {
  const int lane = threadIdx.x % kVG;
  constexpr int kPerWarp = 32 / kVG;
  const int64_t warp = gwarp();
  const int64_t stride = nwarps() * kPerWarp;
  for (int64_t base = warp * kPerWarp; base < a.nv; base += stride) {
    const int64_t v = base + (threadIdx.x & 31) / kVG;
    const bool valid = v < a.nv;
    float ax = 0.f, ay = 0.f, az = 0.f;
    const float wv = valid ? a.invm[v] : 0.0f;
    if (valid && wv != 0.0f) {
      const int32_t k0 = a.inc_ptr[v], k1 = a.inc_ptr[v + 1];
      for (int32_t k = k0 + lane; k < k1; k += kVG) {
        const float4 e = __ldg(a.gV + k);
        const int32_t t = __float_as_int(e.w);
        const float xt = a.z[t] + b.fb[__ldg(b.cbody + t)] * a.p[t];
        ax += xt * e.x;
        ay += xt * e.y;
        az += xt * e.z;
      }
    }
#pragma unroll
    for (int o = kVG / 2; o > 0; o >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, o, kVG);
      ay += __shfl_xor_sync(0xffffffffu, ay, o, kVG);
      az += __shfl_xor_sync(0xffffffffu, az, o, kVG);
    }
    if (valid && lane == 0) a.u[v] = make_float4(wv * ax, wv * ay, wv * az, 0.0f);
  }
}

__global__ void __launch_bounds__(kPT, 2) k_jcg_bodies(PArgs a, BodyCg b) {
  if (a.ctl && a.ctl->skip) return;
  __shared__ float s_c1[kMaxCheb], s_c2[kMaxCheb];
  __shared__ int32_t warm, maxiter;
  __shared__ double tol_abs;
  __shared__ uint32_t status;  // this block's status bits
  __shared__ int s_all;        // every body has stopped
  if (threadIdx.x < kMaxCheb) {
    s_c1[threadIdx.x] = a.js->cf.c1[threadIdx.x];
    s_c2[threadIdx.x] = a.js->cf.c2[threadIdx.x];
  }
  if (threadIdx.x == 0) {
    status = 0;
    warm = a.ctl ? a.ctl->warm : a.warm;
    maxiter = a.ctl ? a.ctl->maxiter : a.maxiter;
    tol_abs = a.ctl ? a.ctl->tol_abs : a.tol_abs;
  }
  const float it = a.js->cf.inv_theta;
  const int m = a.degree;
  const int lane = threadIdx.x & 31;
  unsigned long long gen = 0;
  Own o;
  o.tbeg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  o.tend = a.ta.nt;
  o.tstep = (int64_t)gridDim.x * blockDim.x;
  o.tb0 = 0;
  o.vb0 = 0;
  o.nvb = 0;
  o.e = nullptr;
  o.q = nullptr;
  o.off = nullptr;
  o.w = nullptr;
  __syncthreads();
  // every block reads whether all bodies have stopped after a barrier
  auto all_stopped = [&]() {
    if (threadIdx.x == 0) s_all = ld_relaxed(b.ndone) >= (unsigned int)b.nb;
    __syncthreads();
    return s_all != 0;
  };

  // x = 0 (or the warm start), r = b - A x, p = 0, z = d = D^-1 r / theta;
  // chunk partials of b.b, r.z and r.r
  if (warm) {
    vphase_warm<false>(a, o);
    if (!grid_sync(a, gen)) return;
  }
  for (int64_t c = gwarp(); c < b.nch; c += nwarps()) {
    const int2 r = __ldg(b.ch + c);
    float bb = 0.0f, bz = 0.0f, br = 0.0f;
    for (int64_t t = r.x + lane; t < r.y; t += 32) {
      const float bt = a.b[t];
      float rt = bt;
      if (warm) {
        rt = (float)((double)bt - tdot_warm<false>(a, o, t));
      } else {
        a.x[t] = 0.0f;
      }
      a.xc[t] = 0.0f;
      a.r[t] = rt;
      a.p[t] = 0.0f;
      const float zt = dinv_of<false>(a, t) * rt * it;
      a.z[t] = zt;
      a.d[t] = zt;
      bb += bt * bt;
      bz += rt * zt;
      br += rt * rt;
    }
    const double sb = warp_sum_d(bb), sz = warp_sum_d(bz), sr = warp_sum_d(br);
    if (lane == 0) {
      b.cp[c] = sb;
      b.cp[b.nch + c] = sz;
      b.cp[2LL * b.nch + c] = sr;
    }
  }
  if (!grid_sync(a, gen)) return;
  // per body: |b|^2, r.z, the bound, whether it starts stopped
  for (int64_t k = gwarp(); k < b.nb; k += nwarps()) {
    const double sb = body_total(b, 0, k), sz = body_total(b, 1, k), sr = body_total(b, 2, k);
    if (lane == 0) {
      double* sc = b.sc;
      const double t2 = tol_abs * tol_abs, r2 = a.tol_rel * a.tol_rel * sb;
      const double tol2 = r2 > t2 ? r2 : t2;
      const double rr = warm ? sr : sb;
      // a body with b = 0 (its Newton loop has ended) has x = 0 exactly
      int stop = maxiter <= 0 || (warm && rr < tol2) || sb == 0.0;
      if (!isfinite(sb)) {
        atomicOr(&status, (uint32_t)MGPBD_STATUS_NAN);
        stop = 1;
      }
      sc[0 * b.nb + k] = sb;   // |b|^2
      sc[1 * b.nb + k] = sz;   // r.z
      sc[2 * b.nb + k] = rr;   // r.r
      sc[4 * b.nb + k] = tol2;
      b.fa[k] = 0.0f;
      b.fb[k] = 0.0f;
      b.iters[k] = 0;
      b.done[k] = stop;
      if (stop) atomicAdd(b.ndone, 1u);
    }
  }
  if (!grid_sync(a, gen)) return;
  bool finished = all_stopped();

  // the Chebyshev steps of z = M^-1 r, the last one with chunked partials
  // of r.z into plane 2
  auto cheb_steps = [&]() -> bool {
    for (int i = 1; i < m; ++i) {
      vphase<kSrcX, false>(a, o, 0.0f, a.z);
      if (!grid_sync(a, gen)) return false;
      if (i < m - 1) {
        tphase_cheb<false, false>(a, o, s_c1[i], s_c2[i], nullptr);
      } else {
        const float c1 = s_c1[i], c2 = s_c2[i];
        for (int64_t c = gwarp(); c < b.nch; c += nwarps()) {
          const int2 r = __ldg(b.ch + c);
          float acc = 0.0f;
          for (int64_t tb = r.x + lane; tb < r.y; tb += 32 * kTB) {
            float y[kTB];
#pragma unroll
            for (int q = 0; q < kTB; ++q) {
              const int64_t t = tb + 32 * q;
              y[q] = t < r.y ? tdot_any<false>(a, o, t) : 0.0f;
            }
#pragma unroll
            for (int q = 0; q < kTB; ++q) {
              const int64_t t = tb + 32 * q;
              if (t < r.y) {
                const float zt = a.z[t];
                const float yt = y[q] + __ldg(a.ta.alpha + t) * zt;
                const float rt = a.r[t];
                const float rrv = dinv_of<false>(a, t) * (rt - yt);
                const float dt = c1 * a.d[t] + c2 * rrv;
                a.d[t] = dt;
                const float zn = zt + dt;
                a.z[t] = zn;
                acc += rt * zn;
              }
            }
          }
          const double s = warp_sum_d(acc);
          if (lane == 0) b.cp[2LL * b.nch + c] = s;
        }
      }
      if (!grid_sync(a, gen)) return false;
    }
    return true;
  };

  if (!finished && m > 1) {
    if (!cheb_steps()) return;
    for (int64_t k = gwarp(); k < b.nb; k += nwarps()) {
      const double sz = body_total(b, 2, k);
      if (lane == 0 && !b.done[k]) {
        b.sc[1 * b.nb + k] = sz;
        if (!isfinite(sz)) {
          atomicOr(&status, (uint32_t)MGPBD_STATUS_NAN);
          b.done[k] = 1;
          atomicAdd(b.ndone, 1u);
        }
      }
    }
    if (!grid_sync(a, gen)) return;
    finished = all_stopped();
  }

  int32_t iters = 0;
  while (!finished) {
    // u = W J^T (z + beta_b p)
    vphase_body_zbp(a, b);
    if (!grid_sync(a, gen)) return;
    // p = z + beta_b p; ap = A p; chunk partials of p.Ap (stopped bodies
    // skipped)
    for (int64_t c = gwarp(); c < b.nch; c += nwarps()) {
      const int2 r = __ldg(b.ch + c);
      const int32_t k = __ldg(b.chb + c);
      if (b.done[k]) continue;
      const float bf = b.fb[k];
      float acc = 0.0f;
      for (int64_t tb = r.x + lane; tb < r.y; tb += 32 * kTB) {
        float y[kTB];
#pragma unroll
        for (int q = 0; q < kTB; ++q) {
          const int64_t t = tb + 32 * q;
          y[q] = t < r.y ? tdot_any<false>(a, o, t) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < kTB; ++q) {
          const int64_t t = tb + 32 * q;
          if (t < r.y) {
            const float pt = a.z[t] + bf * a.p[t];
            const float yt = y[q] + __ldg(a.ta.alpha + t) * pt;
            a.p[t] = pt;
            a.ap[t] = yt;
            acc += pt * yt;
          }
        }
      }
      const double s = warp_sum_d(acc);
      if (lane == 0) b.cp[c] = s;
    }
    if (!grid_sync(a, gen)) return;
    // body alphas
    for (int64_t k = gwarp(); k < b.nb; k += nwarps()) {
      if (b.done[k]) continue;  // warp-uniform
      const double pap = body_total(b, 0, k);
      if (lane == 0) {
        b.sc[3 * b.nb + k] = pap;
        if (!isfinite(pap)) atomicOr(&status, (uint32_t)MGPBD_STATUS_NAN);
        if (!(fabs(pap) >= 1e-30) || !isfinite(pap)) {
          b.done[k] = 1;
          b.fa[k] = 0.0f;
          atomicAdd(b.ndone, 1u);
        } else {
          if (pap <= 0.0) atomicOr(&status, (uint32_t)MGPBD_STATUS_PAP_NONPOS);
          b.fa[k] = (float)(b.sc[1 * b.nb + k] / pap);
        }
      }
    }
    if (!grid_sync(a, gen)) return;
    // x += alpha_b p (compensated); r -= alpha_b Ap; z = d = D^-1 r / theta;
    // chunk partials of r.r (plane 1) and, degree 1, r.z (plane 2)
    for (int64_t c = gwarp(); c < b.nch; c += nwarps()) {
      const int2 r = __ldg(b.ch + c);
      const int32_t k = __ldg(b.chb + c);
      if (b.done[k]) continue;
      const float al = b.fa[k];
      float acc_rr = 0.0f, acc_rz = 0.0f;
      for (int64_t t = r.x + lane; t < r.y; t += 32) {
        const float pt = a.p[t], apt = a.ap[t];
        const float s = a.x[t];
        const float y = al * pt - a.xc[t];
        const float sn = s + y;
        a.xc[t] = (sn - s) - y;
        a.x[t] = sn;
        const float rt = a.r[t] - al * apt;
        a.r[t] = rt;
        const float zt = dinv_of<false>(a, t) * rt * it;
        a.z[t] = zt;
        a.d[t] = zt;
        acc_rr += rt * rt;
        acc_rz += rt * zt;
      }
      const double srr = warp_sum_d(acc_rr), srz = warp_sum_d(acc_rz);
      if (lane == 0) {
        b.cp[b.nch + c] = srr;
        if (m == 1) b.cp[2LL * b.nch + c] = srz;
      }
    }
    if (!grid_sync(a, gen)) return;
    // body residuals and stopping tests
    for (int64_t k = gwarp(); k < b.nb; k += nwarps()) {
      if (b.done[k]) continue;
      const double rr = body_total(b, 1, k);
      if (lane == 0) {
        b.sc[2 * b.nb + k] = rr;
        int stop = 0;
        if (!isfinite(rr)) {
          atomicOr(&status, (uint32_t)MGPBD_STATUS_NAN);
          stop = 1;
        } else if (rr < b.sc[4 * b.nb + k]) {
          b.iters[k] += 1;
          stop = 1;
        }
        if (stop) {
          b.done[k] = 1;
          atomicAdd(b.ndone, 1u);
        }
      }
    }
    if (!grid_sync(a, gen)) return;
    iters += 1;
    if (all_stopped()) break;
    // (the barrier between every block's read of the stopped count and the
    // next change of it: the Chebyshev steps' own, or one for degree 1)
    if (m > 1) {
      if (!cheb_steps()) return;
    } else if (!grid_sync(a, gen)) {
      return;
    }
    // body betas
    for (int64_t k = gwarp(); k < b.nb; k += nwarps()) {
      if (b.done[k]) continue;
      const double sz = body_total(b, 2, k);
      if (lane == 0) {
        b.iters[k] += 1;
        const double rz = b.sc[1 * b.nb + k];
        int stop = 0;
        if (fabs(rz) < 1e-30) {
          stop = 1;
        } else {
          b.fb[k] = (float)(sz / rz);
          b.sc[1 * b.nb + k] = sz;
          if (b.iters[k] >= maxiter) {
            atomicOr(&status, (uint32_t)MGPBD_STATUS_CG_MAXITER);
            stop = 1;
          }
        }
        if (stop) {
          b.done[k] = 1;
          atomicAdd(b.ndone, 1u);
        }
      }
    }
    if (!grid_sync(a, gen)) return;
    finished = all_stopped();
  }

  // the compensated sums, rounded once (xc keeps what the rounding dropped)
  for (int64_t t = o.tbeg; t < o.tend; t += o.tstep) {
    const float s = a.x[t], c = a.xc[t];
    const float hi = s - c;
    a.xc[t] = (s - hi) - c;
    a.x[t] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    CgState* st = a.st;
    if (status) atomicOr(reinterpret_cast<unsigned int*>(&st->status), status);
    if (blockIdx.x == 0) {
      st->iters = iters;
      st->done = 1;
      st->maxiter = maxiter;
      st->body_runs = 1;
    }
  }
}

int64_t staged_smem_bytes(int32_t emax, int32_t tmax, int32_t vmax) {
  const int64_t b = 16LL * (emax + vmax) + 16LL * tmax + 4LL * (vmax + 1) + 4LL * vmax;
  return (b + 15) / 16 * 16;
}

}  // namespace

JcgPlan jcg_plan(const std::vector<int32_t>& inc_ptr, int32_t nv, int32_t nt, bool allow_staged) {
  require(static_cast<int64_t>(inc_ptr.size()) == static_cast<int64_t>(nv) + 1, MGPBD_EINVAL,
          "incidence offsets must hold nv + 1 entries");
  int dev = 0, coop = 0, sms = 0, optin = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  require(coop != 0, MGPBD_ENOTSUP, "device does not support cooperative launch");
  MGPBD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int64_t ne = inc_ptr[nv];
  if (allow_staged) {
    JcgPlan p;
    const int G = sms;
    p.vb.resize(G + 1);
    p.tb.resize(G + 1);
    // vertices: equal shares of (incident entries + kVertexCost per vertex),
    // so neither gathers nor vertex rounds pile up in one block; tets: equal
    // 32-aligned shares
    const int64_t total = ne + static_cast<int64_t>(kVertexCost) * nv;
    int32_t v = 0;
    for (int b = 0; b <= G; ++b) {
      if (b == G) {
        p.vb[b] = nv;
      } else {
        const int64_t target = total * b / G;
        while (v < nv && inc_ptr[v] + static_cast<int64_t>(kVertexCost) * v < target) ++v;
        p.vb[b] = v;
      }
      const int64_t tt = (static_cast<int64_t>(nt) * b / G + 31) / 32 * 32;
      p.tb[b] = b == G ? nt : static_cast<int32_t>(std::min<int64_t>(tt, nt));
    }
    for (int b = 0; b < G; ++b) {
      p.vmax = std::max(p.vmax, p.vb[b + 1] - p.vb[b]);
      p.tmax = std::max(p.tmax, p.tb[b + 1] - p.tb[b]);
      p.emax = std::max(p.emax, inc_ptr[p.vb[b + 1]] - inc_ptr[p.vb[b]]);
    }
    const int64_t smem = staged_smem_bytes(p.emax, p.tmax, p.vmax);
    if (smem <= optin) {
      MGPBD_CUDA(cudaFuncSetAttribute(k_jcg<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)));
      int occ = 0;
      MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_jcg<true>, kPT,
                                                               static_cast<size_t>(smem)));
      if (occ >= 1) {
        p.staged = true;
        p.grid = G;
        p.smem = static_cast<int>(smem);
        return p;
      }
    }
  }
  // too large to stage: every phase reads from L2, work strided over the grid
  JcgPlan p;
  int occ = 0;
  MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_jcg<false>, kPT, 0));
  require(occ >= 1, MGPBD_ENOTSUP, "persistent CG kernel does not fit on an SM");
  p.staged = false;
  p.grid = sms * occ;
  p.smem = 0;
  return p;
}

// the kernel arguments of one persistent dual CG launch
static PArgs pargs_of(const JView& j, const JcgVecs& v, const JState* js, CgState* st,
                      double tol_abs, double tol_rel, int maxiter, int degree, bool warm,
                      double spin_limit_s, const JcgCtl* ctl) {
  PArgs a;
  a.ta.t_i = reinterpret_cast<const int4*>(j.t_i);
  require(j.gT != nullptr, MGPBD_ESTATE, "persistent CG needs the gradient planes");
  a.ta.gradC = j.gT;
  a.ta.u = j.u;
  a.ta.alpha = j.alpha;
  a.ta.dinv = j.dinv;
  a.unit_dinv = j.unit_dinv ? 1 : 0;
  a.ta.nt = j.nt;
  a.ta.n4 = j.n4;
  a.ta.gE = j.gE;
  a.ta.qE = j.qE;
  require(j.n4 >= j.nt || (j.gE && j.qE), MGPBD_ESTATE, "compact length constraints not prepared");
  a.nv = j.nv;
  a.inc_ptr = j.inc_ptr;
  a.gV = j.gV;
  a.invm = j.invm;
  a.u = j.u;
  a.b = v.b;
  a.x = v.x;
  a.xc = v.xc;
  a.r = v.r;
  a.z = v.z;
  a.d = v.d;
  a.p = v.p;
  a.ap = v.ap;
  a.partials = v.partials;
  a.gs = v.gs;
  a.st = st;
  a.js = js;
  a.part_v = nullptr;
  a.part_t = nullptr;
  a.emax = a.tmax = a.vmax = 0;
  a.tol_abs = tol_abs;
  a.tol_rel = tol_rel;
  a.maxiter = maxiter;
  a.degree = degree;
  a.warm = warm ? 1 : 0;
  a.ulo = v.ulo;
  a.ctl = ctl;
  require(!(warm || ctl) || v.ulo != nullptr, MGPBD_EINVAL, "warm start needs the ulo scratch");
  a.spin_ns = static_cast<unsigned long long>(spin_limit_s * 1e9);
  return a;
}

void launch_jcg_persistent(const JView& j, const JcgVecs& v, const JcgPlan& plan,
                           const int32_t* part_dev, const JState* js, CgState* st, double tol_abs,
                           double tol_rel, int maxiter, int degree, bool warm, double spin_limit_s,
                           cudaStream_t s, const JcgCtl* ctl) {
  require(degree >= 1 && degree <= kMaxCheb, MGPBD_EINVAL, "Chebyshev degree out of range");
  require(plan.grid > 0, MGPBD_ESTATE, "persistent CG plan not built");
  require(3LL * plan.grid <= v.partials_capacity, MGPBD_ERANGE, "partials buffer too small");
  require(!plan.staged || part_dev != nullptr, MGPBD_ESTATE, "staged plan without partition");
  PArgs a = pargs_of(j, v, js, st, tol_abs, tol_rel, maxiter, degree, warm, spin_limit_s, ctl);
  a.part_v = plan.staged ? part_dev : nullptr;
  a.part_t = plan.staged ? part_dev + plan.grid + 1 : nullptr;
  a.emax = plan.emax;
  a.tmax = plan.tmax;
  a.vmax = plan.vmax;
  MGPBD_CUDA(cudaMemsetAsync(v.gs, 0, sizeof(GridSync), s));
  MGPBD_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), s));
  void* args[] = {&a};
  const void* fn = plan.staged ? reinterpret_cast<const void*>(k_jcg<true>)
                               : reinterpret_cast<const void*>(k_jcg<false>);
  // the dynamic shared-memory limit is a per-function attribute shared by
  // every handle in the process: set this plan's before each staged launch
  if (plan.staged)
    MGPBD_CUDA(cudaFuncSetAttribute(k_jcg<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    plan.smem));
  MGPBD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(plan.grid), dim3(kPT), args,
                                         static_cast<size_t>(plan.smem), s));
  MGPBD_CHECK_LAUNCH();
}

void launch_jcg_bodies(const JView& j, const JcgVecs& v, const BodyCg& bc, const JState* js,
                       CgState* st, double tol_abs, double tol_rel, int maxiter, int degree,
                       bool warm, double spin_limit_s, cudaStream_t s, const JcgCtl* ctl) {
  require(degree >= 1 && degree <= kMaxCheb, MGPBD_EINVAL, "Chebyshev degree out of range");
  require(bc.nb > 0 && bc.nch > 0 && bc.ch && bc.chb && bc.bptr && bc.bidx && bc.cbody &&
              bc.cp && bc.sc && bc.fa && bc.fb && bc.done && bc.iters && bc.ndone,
          MGPBD_ESTATE, "per-body CG arrays not prepared");
  PArgs a = pargs_of(j, v, js, st, tol_abs, tol_rel, maxiter, degree, warm, spin_limit_s, ctl);
  int dev = 0, sms = 0, occ = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_jcg_bodies, kPT, 0));
  require(occ >= 1, MGPBD_ESTATE, "per-body CG kernel cannot be resident");
  const int grid = std::min(occ, 2) * sms;
  MGPBD_CUDA(cudaMemsetAsync(v.gs, 0, sizeof(GridSync), s));
  MGPBD_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), s));
  MGPBD_CUDA(cudaMemsetAsync(bc.ndone, 0, sizeof(uint32_t), s));
  BodyCg b = bc;
  void* args[] = {&a, &b};
  MGPBD_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_jcg_bodies), dim3(grid),
                                         dim3(kPT), args, 0, s));
  MGPBD_CHECK_LAUNCH();
}

}  // namespace mgpbd
