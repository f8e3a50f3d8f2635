// Matrix-free A = J W J^T + alpha~ and the Chebyshev-preconditioned CG of
// FAST mode (see jform.cuh).  Reductions finish in the last block of the
// kernel that produces them (ticket counter + fixed-order sum), so one CG
// iteration of degree k is 2k + 2 kernels with no scalar-only launches.
#include "jform.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <unordered_map>

#include "common.h"
#include "jform_dev.cuh"

namespace mgpbd {

namespace {

using namespace jdev;

constexpr int kT = 256;  // threads per block

// ---------------------------------------------------------------------------
__global__ void k_jprep(const int32_t* __restrict__ inc_ent, int64_t ne,
                        const float* __restrict__ gradC, const int4* __restrict__ t_i,
                        const float* __restrict__ invm, const float* __restrict__ alpha,
                        int32_t nt, float4* __restrict__ gV, float* __restrict__ dinv,
                        float4* __restrict__ gT, int32_t n4, float4* __restrict__ gE,
                        int unit_dinv) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ne; k += stride) {
    const int32_t e = inc_ent[k];
    const float* g = gradC + 3LL * e;
    gV[k] = make_float4(g[0], g[1], g[2], __int_as_float(e >> 2));
  }
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += stride) {
    const int4 q = t_i[t];
    const float* g = gradC + 12 * t;
    const float w[4] = {invm[q.x], invm[q.y], invm[q.z], invm[q.w]};
    float d = 0.0f;
#pragma unroll
    for (int l = 0; l < 4; ++l)
      d += w[l] * (g[3 * l] * g[3 * l] + g[3 * l + 1] * g[3 * l + 1] + g[3 * l + 2] * g[3 * l + 2]);
    d += alpha[t];
    dinv[t] = unit_dinv ? 1.0f : (fabsf(d) > 1e-30f ? 1.0f / d : 0.0f);
    if (gT) {
      const float4* g4 = reinterpret_cast<const float4*>(g);
      gT[t] = g4[0];
      gT[nt + t] = g4[1];
      gT[2LL * nt + t] = g4[2];
    }
    if (gE && t >= n4) gE[t - n4] = make_float4(g[0], g[1], g[2], 0.0f);
  }
}

// vertex phase: u_v = w_v sum x_t g_{t,l}, x_t from Src
template <int SRC>
__global__ void __launch_bounds__(kT)
    k_jv(int32_t nv, const int32_t* __restrict__ inc_ptr, const float4* __restrict__ gV,
         const float* __restrict__ invm, const float* __restrict__ x, const float* __restrict__ p,
         const CgState* __restrict__ st, const JState* __restrict__ js, float4* __restrict__ u,
         float scale_unused) {
  if (st && st->done) return;
  float beta = 0.0f;
  if (SRC == kSrcZbP) beta = (float)st->beta;
  const int lane = threadIdx.x % kVG;
  constexpr int kPerWarp = 32 / kVG;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t stride = ((int64_t)gridDim.x * blockDim.x >> 5) * kPerWarp;
  for (int64_t base = warp * kPerWarp; base < nv; base += stride) {
    const int64_t v = base + (threadIdx.x & 31) / kVG;
    const bool valid = v < nv;
    float w;
    const float3 a = jv_group<SRC>(v, valid, lane, inc_ptr, gV, invm, x, p, beta, &w);
    if (valid && lane == 0) u[v] = make_float4(w * a.x, w * a.y, w * a.z, 0.0f);
  }
}

// y = A x (tests)
__global__ void k_jt_plain(TArgs a, const float* __restrict__ x, float* __restrict__ y) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < a.nt;
       t += (int64_t)gridDim.x * blockDim.x)
    y[t] = jt_core(a, t) + a.alpha[t] * x[t];
}

// p = z + beta p; Ap; p.Ap -> alpha (last block)
__global__ void __launch_bounds__(kT)
    k_jt_ap(TArgs a, const float* __restrict__ z, float* __restrict__ p, float* __restrict__ ap,
            double* __restrict__ partials, CgState* st, JState* js) {
  if (st->done) return;
  const float beta = (float)st->beta;
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < a.nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float pt = z[t] + beta * p[t];
    const float y = jt_core(a, t) + a.alpha[t] * pt;
    p[t] = pt;
    ap[t] = y;
    acc += (double)pt * (double)y;
  }
  if (publish_last(acc, partials, &js->ticket[0])) {
    const double pap = gather_partials(partials, gridDim.x);
    if (threadIdx.x == 0) {
      js->ticket[0] = 0;
      st->pap = pap;
      if (!isfinite(pap)) st->status |= MGPBD_STATUS_NAN;
      if (!(fabs(pap) >= 1e-30) || !isfinite(pap)) {
        st->done = 1;
      } else {
        if (pap <= 0.0) st->status |= MGPBD_STATUS_PAP_NONPOS;
        st->alpha = st->rz / pap;
      }
    }
  }
}

// x += alpha p ; r -= alpha Ap ; first Chebyshev step z = d = D^-1 r / theta
__global__ void __launch_bounds__(kT)
    k_ju(int32_t nt, const float* __restrict__ p, const float* __restrict__ ap,
         const float* __restrict__ dinv, double* __restrict__ xd, double* __restrict__ r,
         float* __restrict__ z, float* __restrict__ d, double* __restrict__ partials,
         CgState* st, JState* js) {
  if (st->done) return;
  const double al = st->alpha;
  const float it = js->cf.inv_theta;
  const bool jac = js->cf.degree == 1;
  double rr = 0.0, rz = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    xd[t] += al * (double)p[t];
    const double rt = r[t] - al * (double)ap[t];
    r[t] = rt;
    const float zt = dinv[t] * (float)rt * it;
    z[t] = zt;
    d[t] = zt;
    rr += rt * rt;
    rz += rt * (double)zt;
  }
  // two reductions: r.r (partials[0..G)) and, for degree 1, r.z ([G..2G))
  double* p2 = partials + gridDim.x;
  {
    double v2 = block_sum_d(rz);
    if (threadIdx.x == 0) p2[blockIdx.x] = v2;
  }
  if (publish_last(rr, partials, &js->ticket[1])) {
    const double rrs = gather_partials(partials, gridDim.x);
    const double rzs = jac ? gather_partials(p2, gridDim.x) : 0.0;
    if (threadIdx.x == 0) {
      js->ticket[1] = 0;
      st->rr = rrs;
      if (!isfinite(rrs)) {
        st->status |= MGPBD_STATUS_NAN;
        st->done = 1;
      } else if (rrs < st->tol2) {
        st->iters += 1;
        st->done = 1;
      } else if (jac) {
        st->rz_new = rzs;
        if (fabs(st->rz) < 1e-30) {
          st->iters += 1;
          st->done = 1;
        } else {
          st->beta = rzs / st->rz;
          st->rz = rzs;
          st->iters += 1;
          if (st->iters >= st->maxiter) {
            st->done = 1;
            st->status |= MGPBD_STATUS_CG_MAXITER;
          }
        }
      }
    }
  }
}

// Chebyshev step i >= 1: rr = D^-1 (r - A z); d = c1 d + c2 rr; z += d.
// The last step also reduces r.z: init -> rz; loop -> beta, iteration count.
template <bool LAST, bool INIT>
__global__ void __launch_bounds__(kT)
    k_jt_cheb(TArgs a, int step, const double* __restrict__ r, float* __restrict__ z,
              float* __restrict__ d, double* __restrict__ partials, CgState* st, JState* js) {
  if (st->done) return;
  const float c1 = js->cf.c1[step], c2 = js->cf.c2[step];
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < a.nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float zt = z[t];
    const float y = jt_core(a, t) + a.alpha[t] * zt;
    const float rt = (float)r[t];
    const float rrv = a.dinv[t] * (rt - y);
    const float dt = c1 * d[t] + c2 * rrv;
    d[t] = dt;
    const float zn = zt + dt;
    z[t] = zn;
    if (LAST) acc += r[t] * (double)zn;
  }
  if (!LAST) return;
  if (publish_last(acc, partials, &js->ticket[2])) {
    const double rz = gather_partials(partials, gridDim.x);
    if (threadIdx.x == 0) {
      js->ticket[2] = 0;
      if (INIT) {
        st->rz = rz;
        if (!isfinite(rz)) {
          st->status |= MGPBD_STATUS_NAN;
          st->done = 1;
        }
      } else {
        st->rz_new = rz;
        if (fabs(st->rz) < 1e-30) {
          st->iters += 1;
          st->done = 1;
        } else {
          st->beta = rz / st->rz;
          st->rz = rz;
          st->iters += 1;
          if (st->iters >= st->maxiter) {
            st->done = 1;
            st->status |= MGPBD_STATUS_CG_MAXITER;
          }
        }
      }
    }
  }
}

// CG init: x = 0, r = b, p = 0, z = d = D^-1 b / theta; b.b -> tolerance
__global__ void __launch_bounds__(kT)
    k_ju0(int32_t nt, const float* __restrict__ b, const float* __restrict__ dinv,
          double* __restrict__ xd, double* __restrict__ r, float* __restrict__ z,
          float* __restrict__ d, float* __restrict__ p, double* __restrict__ partials,
          CgState* st, JState* js, double tol_abs, double tol_rel, int maxiter) {
  const float it = js->cf.inv_theta;
  const bool jac = js->cf.degree == 1;
  double bb = 0.0, rz = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float bt = b[t];
    xd[t] = 0.0;
    r[t] = bt;
    p[t] = 0.0f;
    const float zt = dinv[t] * bt * it;
    z[t] = zt;
    d[t] = zt;
    bb += (double)bt * bt;
    rz += (double)bt * zt;
  }
  double* p2 = partials + gridDim.x;
  {
    double v2 = block_sum_d(rz);
    if (threadIdx.x == 0) p2[blockIdx.x] = v2;
  }
  if (publish_last(bb, partials, &js->ticket[3])) {
    const double bbs = gather_partials(partials, gridDim.x);
    const double rzs = gather_partials(p2, gridDim.x);
    if (threadIdx.x == 0) {
      js->ticket[3] = 0;
      st->rr0 = bbs;
      const double t2 = tol_abs * tol_abs, r2 = tol_rel * tol_rel * bbs;
      st->tol2 = r2 > t2 ? r2 : t2;
      st->iters = 0;
      st->maxiter = maxiter;
      st->done = maxiter <= 0;
      st->status = isfinite(bbs) ? 0 : MGPBD_STATUS_NAN;
      st->beta = 0.0;
      st->alpha = st->pap = st->rr = st->rz_new = 0.0;
      st->body_runs = 0;
      st->rz = jac ? rzs : 0.0;
    }
  }
}

__global__ void k_jfinish(const double* __restrict__ xd, float* __restrict__ x, int32_t nt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x)
    x[t] = (float)xd[t];
}

// Lanczos on S = D^-1/2 A D^-1/2 (Golub & Van Loan, sec. 10.1): step j
// computes w = S q_j - b_{j-1} q_{j-1} and a_j = q_j . w ...
__global__ void __launch_bounds__(kT)
    k_lz_apply(TArgs a, int j, const float* __restrict__ q, const float* __restrict__ qprev,
               float* __restrict__ w, double* __restrict__ partials, JState* js) {
  const float bprev = j > 0 ? (float)js->lz_b[j - 1] : 0.0f;
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < a.nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float sd = sqrtf(a.dinv[t]);
    const float y = sd * (jt_core(a, t) + a.alpha[t] * q[t] * sd) - bprev * qprev[t];
    w[t] = y;
    acc += (double)q[t] * y;
  }
  if (publish_last(acc, partials, &js->ticket[0])) {
    const double s = gather_partials(partials, gridDim.x);
    if (threadIdx.x == 0) {
      js->ticket[0] = 0;
      js->lz_a[j] = s;
    }
  }
}

// ... then w -= a_j q_j and b_j = |w|
__global__ void __launch_bounds__(kT)
    k_lz_orth(int32_t nt, int j, const float* __restrict__ q, float* __restrict__ w,
              double* __restrict__ partials, JState* js) {
  const float aj = (float)js->lz_a[j];
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float y = w[t] - aj * q[t];
    w[t] = y;
    acc += (double)y * y;
  }
  if (publish_last(acc, partials, &js->ticket[1])) {
    const double s = gather_partials(partials, gridDim.x);
    if (threadIdx.x == 0) {
      js->ticket[1] = 0;
      js->lz_b[j] = sqrt(s);
    }
  }
}

// q_{j+1} = w / b_j, q_j -> qprev
__global__ void k_lz_next(int32_t nt, int j, float* __restrict__ q, float* __restrict__ qprev,
                          const float* __restrict__ w, const JState* js) {
  const double b = js->lz_b[j];
  const float inv = b > 0.0 ? (float)(1.0 / b) : 0.0f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    qprev[t] = q[t];
    q[t] = w[t] * inv;
  }
}

// start vector: fixed pseudo-random entries, normalised
__global__ void __launch_bounds__(kT)
    k_lz_seed(int32_t nt, float* __restrict__ q, double* __restrict__ partials, JState* js) {
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = static_cast<uint32_t>(t) * 2654435761u;
    h ^= h >> 15;
    const float v = 0.5f + (h & 0xffff) * (1.0f / 65536.0f);
    q[t] = v;
    acc += (double)v * v;
  }
  if (publish_last(acc, partials, &js->ticket[0])) {
    const double s = gather_partials(partials, gridDim.x);
    if (threadIdx.x == 0) {
      js->ticket[0] = 0;
      js->scale = s > 0.0 ? 1.0 / sqrt(s) : 1.0;
    }
  }
}

__global__ void k_lz_scale(int32_t nt, float* __restrict__ q, float* __restrict__ qprev,
                           const JState* js) {
  const float sc = (float)js->scale;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    q[t] *= sc;
    qprev[t] = 0.0f;
  }
}

__global__ void k_seed(float* v, int32_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = static_cast<uint32_t>(i) * 2654435761u;
    h ^= h >> 15;
    v[i] = 0.5f + (h & 0xffff) * (1.0f / 65536.0f);
  }
}

// Blocks of kT threads of `fn` that fit on the device at once (one wave),
// from the occupancy calculator, cached per kernel.  Grids never exceed one
// wave: the kernels stride over their work, so a partial second wave (and
// its tail) never occurs.
int resident_blocks(const void* fn) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(fn);
  if (it != cache.end()) return it->second;
  int dev = 0, sms = 0, per_sm = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  MGPBD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MGPBD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kT, 0));
  int r = std::max(1, std::min(sms * std::max(per_sm, 1), kMaxReduceBlocks));
  cache[fn] = r;
  return r;
}

template <class K>
inline int tgrid_for(K* fn, int64_t n) {
  int64_t g = (n + kT - 1) / kT;
  int cap = resident_blocks(reinterpret_cast<const void*>(fn));
  return static_cast<int>(g < 1 ? 1 : (g > cap ? cap : g));
}

template <class K>
inline int vgrid_for(K* fn, int32_t nv) {
  int64_t g = (static_cast<int64_t>(nv) * kVG + kT - 1) / kT;
  int cap = resident_blocks(reinterpret_cast<const void*>(fn));
  return static_cast<int>(g < 1 ? 1 : (g > cap ? cap : g));
}

// tet-phase grid for kernels whose occupancy is not looked up
inline int tgrid(int64_t n) {
  int64_t g = (n + kT - 1) / kT;
  return static_cast<int>(g < 1 ? 1 : (g > kMaxReduceBlocks ? kMaxReduceBlocks : g));
}

TArgs targs(const JView& j) {
  TArgs a;
  a.t_i = reinterpret_cast<const int4*>(j.t_i);
  a.gradC = reinterpret_cast<const float4*>(j.gradC);
  a.u = j.u;
  a.alpha = j.alpha;
  a.dinv = j.dinv;
  a.nt = j.nt;
  // the per-phase kernels read every constraint's four slots
  a.n4 = j.nt;
  a.gE = nullptr;
  a.qE = nullptr;
  return a;
}

}  // namespace

void launch_jform_prepare(const JView& j, const int32_t* inc_ent, float4* gV, float* dinv,
                          float4* gT, bool unit_dinv, cudaStream_t s) {
  int g = tgrid(std::max<int64_t>(j.ne, j.nt));
  k_jprep<<<g, kT, 0, s>>>(inc_ent, j.ne, j.gradC, reinterpret_cast<const int4*>(j.t_i), j.invm,
                           j.alpha, j.nt, gV, dinv, gT, j.n4, j.gE, unit_dinv ? 1 : 0);
  MGPBD_CHECK_LAUNCH();
}

void launch_jform_apply(const JView& j, const float* x, float* y, cudaStream_t s) {
  k_jv<kSrcX><<<vgrid_for(k_jv<kSrcX>, j.nv), kT, 0, s>>>(j.nv, j.inc_ptr, j.gV, j.invm, x,
                                                            nullptr, nullptr, nullptr, j.u, 0.f);
  MGPBD_CHECK_LAUNCH();
  k_jt_plain<<<tgrid_for(k_jt_plain, j.nt), kT, 0, s>>>(targs(j), x, y);
  MGPBD_CHECK_LAUNCH();
}

void launch_jform_lanczos(const JView& j, float* q, float* qprev, float* w, double* partials,
                          JState* js, int steps, cudaStream_t s) {
  require(steps >= 1 && steps <= kMaxLanczos, MGPBD_EINVAL, "Lanczos steps out of range");
  const int G = tgrid_for(k_lz_apply, j.nt);
  k_lz_seed<<<G, kT, 0, s>>>(j.nt, q, partials, js);
  MGPBD_CHECK_LAUNCH();
  k_lz_scale<<<G, kT, 0, s>>>(j.nt, q, qprev, js);
  MGPBD_CHECK_LAUNCH();
  for (int it = 0; it < steps; ++it) {
    k_jv<kSrcSqrtD><<<vgrid_for(k_jv<kSrcSqrtD>, j.nv), kT, 0, s>>>(j.nv, j.inc_ptr, j.gV, j.invm, q, j.dinv, nullptr,
                                               js, j.u, 0.f);
    MGPBD_CHECK_LAUNCH();
    k_lz_apply<<<G, kT, 0, s>>>(targs(j), it, q, qprev, w, partials, js);
    MGPBD_CHECK_LAUNCH();
    k_lz_orth<<<G, kT, 0, s>>>(j.nt, it, q, w, partials, js);
    MGPBD_CHECK_LAUNCH();
    if (it + 1 < steps) {
      k_lz_next<<<G, kT, 0, s>>>(j.nt, it, q, qprev, w, js);
      MGPBD_CHECK_LAUNCH();
    }
  }
}

// Number of eigenvalues of the symmetric tridiagonal T (diagonal a,
// off-diagonal b, k rows) below x: the sign changes of the Sturm sequence.
__device__ int sturm_below(const double* a, const double* b, int k, double x) {
  int c = 0;
  double d = 1.0;
  for (int i = 0; i < k; ++i) {
    const double q = i > 0 ? __ddiv_rn(__dmul_rn(b[i - 1], b[i - 1]), d) : 0.0;
    d = (a[i] - x) - q;
    if (d == 0.0) d = -1e-300;
    if (d < 0.0) ++c;
  }
  return c;
}

// Largest eigenvalue of T by Sturm multisection on its Gershgorin interval,
// one warp: each round the 32 lanes count the eigenvalues below 32 points
// that split the interval into 33 parts, and the interval shrinks to the
// part that holds the largest eigenvalue (the first point with all k below
// it is the new upper end), until its width is below 1e-12 of the upper
// end.  Every product that feeds a sum is rounded on its own (no fused
// multiply-add).  The result is the upper end, in all lanes.
__device__ double lanczos_lmax(const double* a, const double* b, int k) {
  const int lane = threadIdx.x & 31;
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < k; ++i) {
    const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < k ? fabs(b[i]) : 0.0);
    lo = fmin(lo, a[i] - r);
    hi = fmax(hi, a[i] + r);
  }
  if (!(hi >= lo) || !isfinite(hi) || !isfinite(lo)) return NAN;
  for (int it = 0; it < 60 && hi - lo > __dmul_rn(1e-12, fmax(1.0, fabs(hi))); ++it) {
    const double step = __ddiv_rn(hi - lo, 33.0);
    const double x = lane == 31 ? hi - step : lo + __dmul_rn(step, static_cast<double>(lane + 1));
    const unsigned all = __ballot_sync(0xffffffffu, sturm_below(a, b, k, x) >= k);
    // the first point with every eigenvalue below it bounds the largest;
    // none: the largest lies above the last point
    const int f = all ? __ffs(all) - 1 : 32;
    const double nlo = f == 0 ? lo : __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
    const double nhi = f == 32 ? hi : __shfl_sync(0xffffffffu, x, f < 32 ? f : 31);
    lo = nlo;
    hi = nhi;
  }
  return hi;
}

// Chebyshev acceleration coefficients on [hi * lo_ratio, hi] (Saad,
// "Iterative Methods for Sparse Linear Systems", 2nd ed., Alg. 12.1):
// sigma = theta / delta, rho_0 = 1 / sigma, rho_i = 1 / (2 sigma - rho_{i-1}),
// d_i = rho_i rho_{i-1} d_{i-1} + (2 rho_i / delta) r_i.  One warp finds
// lmax; its lane 0 writes the coefficients.
__global__ void k_cheb_coefficients(JState* js, int steps, int degree, double lo_ratio,
                                    uint32_t* status) {
  const double lmax = lanczos_lmax(js->lz_a, js->lz_b, steps);
  if (threadIdx.x != 0) return;
  const bool ok = isfinite(lmax) && lmax > 0.0;
  if (!ok && status) atomicOr(reinterpret_cast<unsigned int*>(status), MGPBD_STATUS_NAN);
  ChebCoef& c = js->cf;
  const double hi = ok ? __dmul_rn(1.02, lmax) : 2.0;
  const double lo = __dmul_rn(hi, lo_ratio);
  const double theta = __dmul_rn(0.5, hi + lo), delta = __dmul_rn(0.5, hi - lo);
  const double sigma = __ddiv_rn(theta, delta);
  double rho = __ddiv_rn(1.0, sigma);
  for (int i = 0; i < kMaxCheb; ++i) {
    c.c1[i] = 0.0f;
    c.c2[i] = 0.0f;
  }
  for (int i = 1; i < degree && i < kMaxCheb; ++i) {
    const double rn = __ddiv_rn(1.0, __dmul_rn(2.0, sigma) - rho);
    c.c1[i] = static_cast<float>(__dmul_rn(rn, rho));
    c.c2[i] = static_cast<float>(__ddiv_rn(__dmul_rn(2.0, rn), delta));
    rho = rn;
  }
  c.theta = theta;
  c.lmax = ok ? lmax : (isfinite(lmax) ? lmax : NAN);
  c.inv_theta = static_cast<float>(__ddiv_rn(1.0, theta));
  c.degree = degree;
}

void launch_cheb_coefficients(JState* js, int steps, int degree, double lo_ratio,
                              uint32_t* status, cudaStream_t s) {
  require(steps >= 1 && steps <= kMaxLanczos, MGPBD_EINVAL, "Lanczos steps out of range");
  k_cheb_coefficients<<<1, 32, 0, s>>>(js, steps, degree, lo_ratio, status);
  MGPBD_CHECK_LAUNCH();
}

void launch_jcg_init(const JView& j, const JVecs& v, JState* js, CgState* st, double tol_abs,
                     double tol_rel, int maxiter, cudaStream_t s) {
  const int G = tgrid_for(k_ju0, j.nt);
  k_ju0<<<G, kT, 0, s>>>(j.nt, v.b, j.dinv, v.xd, v.r, v.z, v.d, v.p, v.partials, st, js, tol_abs,
                         tol_rel, maxiter);
  MGPBD_CHECK_LAUNCH();
  // remaining Chebyshev steps of z = M^-1 r (degree read on the host side
  // from the same value given to launch_jform_cheb_setup)
}

void launch_jcg_cheb_steps(const JView& j, const JVecs& v, JState* js, CgState* st, int degree,
                           bool init, cudaStream_t s) {
  const int G = tgrid_for(k_jt_cheb<true, false>, j.nt);
  for (int i = 1; i < degree; ++i) {
    k_jv<kSrcX><<<vgrid_for(k_jv<kSrcX>, j.nv), kT, 0, s>>>(j.nv, j.inc_ptr, j.gV, j.invm, v.z, nullptr, st, js, j.u,
                                            0.f);
    MGPBD_CHECK_LAUNCH();
    const bool last = i == degree - 1;
    if (last && init)
      k_jt_cheb<true, true><<<G, kT, 0, s>>>(targs(j), i, v.r, v.z, v.d, v.partials, st, js);
    else if (last)
      k_jt_cheb<true, false><<<G, kT, 0, s>>>(targs(j), i, v.r, v.z, v.d, v.partials, st, js);
    else
      k_jt_cheb<false, false><<<G, kT, 0, s>>>(targs(j), i, v.r, v.z, v.d, v.partials, st, js);
    MGPBD_CHECK_LAUNCH();
  }
}

void launch_jcg_body(const JView& j, const JVecs& v, JState* js, CgState* st, int degree,
                     cudaStream_t s) {
  k_jv<kSrcZbP><<<vgrid_for(k_jv<kSrcZbP>, j.nv), kT, 0, s>>>(j.nv, j.inc_ptr, j.gV, j.invm, v.z,
                                                              v.p, st, js, j.u, 0.f);
  MGPBD_CHECK_LAUNCH();
  k_jt_ap<<<tgrid_for(k_jt_ap, j.nt), kT, 0, s>>>(targs(j), v.z, v.p, v.ap, v.partials, st, js);
  MGPBD_CHECK_LAUNCH();
  k_ju<<<tgrid_for(k_ju, j.nt), kT, 0, s>>>(j.nt, v.p, v.ap, j.dinv, v.xd, v.r, v.z, v.d, v.partials, st, js);
  MGPBD_CHECK_LAUNCH();
  launch_jcg_cheb_steps(j, v, js, st, degree, false, s);
}

void launch_jcg_finish(const JVecs& v, int32_t nt, const CgState* st, cudaStream_t s) {
  (void)st;
  k_jfinish<<<tgrid(nt), kT, 0, s>>>(v.xd, v.x, nt);
  MGPBD_CHECK_LAUNCH();
}

void launch_seed(float* v, int32_t n, cudaStream_t s) {
  k_seed<<<tgrid(n), kT, 0, s>>>(v, n);
  MGPBD_CHECK_LAUNCH();
}

}  // namespace mgpbd
