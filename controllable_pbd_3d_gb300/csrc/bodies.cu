// Device-side decisions of the packed-body Newton loop (see bodies.cuh).
// Each kernel is one block; per-body work is strided over its threads, the
// loop-wide values are formed by thread 0 in body order (the host loop's
// order).  Products that feed sums are rounded on their own (no fused
// multiply-add), as the host compiles them.
#include <cuda_runtime.h>

#include <algorithm>

#include "bodies.cuh"

namespace mgpbd {
namespace {

constexpr int kBT = 256;

// sum of the chunk partials of group g of body k, chunks ascending
__device__ __forceinline__ double body_sum(const BodyArrays& ba, int32_t k, int g) {
  double acc = 0.0;
  const double* p = ba.partials + static_cast<int64_t>(g) * ba.n_chunks;
  for (int32_t q = ba.chunk_ptr[k]; q < ba.chunk_ptr[k + 1]; ++q) acc += p[ba.chunk_idx[q]];
  return acc;
}

__global__ void __launch_bounds__(kBT) k_bodies_reset(BodyArrays ba, BodyLoop* L) {
  if (threadIdx.x == 0) {
    BodyLoop z{};
    z.omega_min = 1.0;
    *L = z;
  }
  for (int32_t k = threadIdx.x; k < ba.nb; k += blockDim.x) {
    ba.active[k] = 1;
    ba.newton[k] = 0;
    ba.omega_h[k] = 1.0;
  }
}

__global__ void __launch_bounds__(kBT)
    k_bodies_residual(BodyArrays ba, BodyLoop* L, BodyLimits lim,
                      cudaGraphConditionalHandle handle) {
  __shared__ int s_ite, s_end, s_nact;
  if (threadIdx.x == 0) {
    s_ite = L->ite;
    s_end = L->ite >= lim.maxiter || (L->status & MGPBD_STATUS_SYNC_TIMEOUT) != 0;
    s_nact = 0;
  }
  __syncthreads();
  if (s_end) {
    if (threadIdx.x == 0) {
      L->go = 0;
      cudaGraphSetConditional(handle, 0u);
    }
    return;
  }
  const int ite = s_ite;
  for (int32_t k = threadIdx.x; k < ba.nb; k += blockDim.x) ba.sq[k] = body_sum(ba, k, 0);
  __syncthreads();
  if (threadIdx.x == 0) {
    double rg2 = 0.0;
    for (int32_t k = 0; k < ba.nb; ++k) rg2 += ba.sq[k];
    const double r = sqrt(rg2);
    if (ite == 0) L->residual0 = r;
    L->residual = r;
    if (!isfinite(r)) {
      L->status |= MGPBD_STATUS_NAN;
      s_end = 1;
    }
  }
  __syncthreads();
  if (s_end) {
    if (threadIdx.x == 0) {
      L->go = 0;
      cudaGraphSetConditional(handle, 0u);
    }
    return;
  }
  for (int32_t k = threadIdx.x; k < ba.nb; k += blockDim.x) {
    ba.bnorm[k] = 0.0;
    if (ite == 0) ba.r0[k] = sqrt(ba.sq[k]);
    if (!ba.active[k]) continue;
    const double rk = sqrt(ba.sq[k]);
    ba.r[k] = rk;
    if (rk < static_cast<double>(lim.atol) ||
        (ba.r0[k] > 1e-12 && rk < __dmul_rn(static_cast<double>(lim.rtol), ba.r0[k]))) {
      ba.active[k] = 0;
    } else {
      ba.bnorm[k] = rk;
      atomicAdd(&s_nact, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int go = s_nact > 0;
    if (!go) {
      if (ite < ba.log_cap) ba.log[ite] = BodyLogEntry{L->residual, 0.0, 1.0};
      L->n_log = ite + 1;
    } else {
      double bn2 = 0.0;
      for (int32_t k = 0; k < ba.nb; ++k) bn2 = __dadd_rn(bn2, __dmul_rn(ba.bnorm[k], ba.bnorm[k]));
      const double tol = fmax(static_cast<double>(lim.tol_cg),
                              __dmul_rn(static_cast<double>(lim.rel_tol_cg), sqrt(bn2)));
      L->pass = 0;
      L->cg_newton = 0;
      L->left = lim.maxiter_cg;
      // per-body CG: each body's bound is max(tol_cg, rel_tol_cg |b_b|), the
      // kernel's own test
      L->jc.tol_abs = lim.per_body_cg ? static_cast<double>(lim.tol_cg) : tol;
      L->jc.maxiter = lim.maxiter_cg;
      L->jc.warm = 0;
      L->jc.skip = 0;
      if (lim.maxiter_cg <= 0) {  // no pass runs
        L->jc.skip = 1;
        L->status |= MGPBD_STATUS_CG_MAXITER;
      }
    }
    L->go = go;
    cudaGraphSetConditional(handle, go ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(kBT)
    k_bodies_verify(BodyArrays ba, BodyLoop* L, const CgState* st, BodyLimits lim) {
  __shared__ int s_skip;
  __shared__ double s_min[kBT];
  if (threadIdx.x == 0) {
    s_skip = L->jc.skip;
    if (!s_skip) {
      const int32_t its = st->iters;
      const uint32_t stv = static_cast<uint32_t>(st->status);
      L->cg_newton += its;
      L->left -= its;
      L->cg_launches += 1;
      L->status |= stv;
      if (stv & MGPBD_STATUS_SYNC_TIMEOUT) {
        L->jc.skip = 1;
        s_skip = 1;
      } else if (stv & (MGPBD_STATUS_NAN | MGPBD_STATUS_PAP_NONPOS)) {
        L->status |= MGPBD_STATUS_CG_MAXITER;
        L->jc.skip = 1;
        s_skip = 1;
      }
    }
  }
  __syncthreads();
  if (s_skip) return;
  if (lim.per_body_cg) {  // the kernel tested every body against its own bound
    if (threadIdx.x == 0) L->jc.skip = 1;
    return;
  }
  double need = INFINITY;
  for (int32_t k = threadIdx.x; k < ba.nb; k += blockDim.x) {
    const double bound = fmax(static_cast<double>(lim.tol_cg),
                              __dmul_rn(static_cast<double>(lim.rel_tol_cg), ba.bnorm[k]));
    if (ba.bnorm[k] > 0.0 && sqrt(body_sum(ba, k, 0)) > bound) need = fmin(need, bound);
  }
  s_min[threadIdx.x] = need;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < blockDim.x; ++i) need = fmin(need, s_min[i]);
    if (!(need < INFINITY)) {
      L->jc.skip = 1;  // every body meets its bound
    } else {
      L->pass += 1;
      if (L->pass >= 6 || L->left <= 0) {
        L->status |= MGPBD_STATUS_CG_MAXITER;
        L->jc.skip = 1;
      } else {
        L->jc.tol_abs = need;
        L->jc.maxiter = L->left;
        L->jc.warm = 1;
      }
    }
  }
}

__global__ void __launch_bounds__(kBT) k_bodies_cur(BodyArrays ba) {
  for (int32_t k = threadIdx.x; k < ba.nb; k += blockDim.x) ba.cur[k] = body_sum(ba, k, 0);
}

__global__ void __launch_bounds__(kBT)
    k_bodies_omega(BodyArrays ba, BodyLoop* L, BodyLimits lim, int n_trials) {
  __shared__ double s_min[kBT];
  double om_min = 1.0;
  for (int32_t k = threadIdx.x; k < ba.nb; k += blockDim.x) {
    float om = 1.0f;
    if (ba.active[k]) {
      double w = ldexp(1.0, -n_trials);
      const double c = sqrt(ba.cur[k]);
      for (int q = 0; q < n_trials; ++q)
        if (sqrt(body_sum(ba, k, q)) < c) {
          w = ldexp(1.0, -q);
          break;
        }
      om = static_cast<float>(w);
      ba.newton[k] += 1;
      ba.omega_h[k] = om;
      om_min = fmin(om_min, static_cast<double>(om));
    }
    ba.omega[k] = om;
  }
  s_min[threadIdx.x] = om_min;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < blockDim.x; ++i) om_min = fmin(om_min, s_min[i]);
    const int ite = L->ite;
    if (ite < ba.log_cap)
      ba.log[ite] = BodyLogEntry{L->residual, static_cast<double>(L->cg_newton), om_min};
    L->n_log = ite + 1;
    L->omega_min = om_min;
    L->cg_total += L->cg_newton;
    if (ite + 1 == lim.maxiter) L->status |= MGPBD_STATUS_NEWTON_MAXITER;
    L->ite = ite + 1;
  }
}

__global__ void k_bodies_warm_in(BodyLoop* L, const int32_t* have_prev, float* x,
                                 const float* prev, int32_t n) {
  if (L->ite != 0 || !*have_prev) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = prev[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) L->jc.warm = 1;
}

__global__ void k_bodies_warm_out(const BodyLoop* L, int32_t* have_prev, const float* x,
                                  float* prev, int32_t n) {
  if (L->ite != 0 || (L->status & (MGPBD_STATUS_NAN | MGPBD_STATUS_CG_MAXITER))) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    prev[i] = x[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) *have_prev = 1;
}

}  // namespace

void launch_bodies_warm_in(BodyLoop* L, const int32_t* have_prev, float* x, const float* prev,
                           int32_t n, cudaStream_t s) {
  k_bodies_warm_in<<<std::max(1, std::min((n + kBT - 1) / kBT, 4096)), kBT, 0, s>>>(L, have_prev, x,
                                                                                 prev, n);
  MGPBD_CHECK_LAUNCH();
}

void launch_bodies_warm_out(const BodyLoop* L, int32_t* have_prev, const float* x, float* prev,
                            int32_t n, cudaStream_t s) {
  k_bodies_warm_out<<<std::max(1, std::min((n + kBT - 1) / kBT, 4096)), kBT, 0, s>>>(L, have_prev,
                                                                                  x, prev, n);
  MGPBD_CHECK_LAUNCH();
}

void launch_bodies_reset(const BodyArrays& ba, BodyLoop* L, cudaStream_t s) {
  k_bodies_reset<<<1, kBT, 0, s>>>(ba, L);
  MGPBD_CHECK_LAUNCH();
}

void launch_bodies_residual(const BodyArrays& ba, BodyLoop* L, const BodyLimits& lim,
                            cudaGraphConditionalHandle handle, cudaStream_t s) {
  k_bodies_residual<<<1, kBT, 0, s>>>(ba, L, lim, handle);
  MGPBD_CHECK_LAUNCH();
}

void launch_bodies_verify(const BodyArrays& ba, BodyLoop* L, const CgState* st,
                          const BodyLimits& lim, cudaStream_t s) {
  k_bodies_verify<<<1, kBT, 0, s>>>(ba, L, st, lim);
  MGPBD_CHECK_LAUNCH();
}

void launch_bodies_cur(const BodyArrays& ba, cudaStream_t s) {
  k_bodies_cur<<<1, kBT, 0, s>>>(ba);
  MGPBD_CHECK_LAUNCH();
}

void launch_bodies_omega(const BodyArrays& ba, BodyLoop* L, const BodyLimits& lim, int n_trials,
                         cudaStream_t s) {
  require(n_trials >= 1 && n_trials <= 30, MGPBD_EINVAL, "line-search trials out of range");
  k_bodies_omega<<<1, kBT, 0, s>>>(ba, L, lim, n_trials);
  MGPBD_CHECK_LAUNCH();
}

}  // namespace mgpbd
