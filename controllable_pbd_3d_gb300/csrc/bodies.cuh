// Device-side control of the packed-body Newton loop (bodies.cu), for the
// substep that runs as one captured CUDA graph: the per-body residuals,
// stopping tests, CG pass tolerances and line-search steps that the host
// loop (Solver::solve_bodies) decides between its launches are decided by
// these single-block kernels instead, with the same arithmetic in the same
// order, so both loops take the same decisions and give the same positions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.h"
#include "jform.cuh"

namespace mgpbd {

// Loop state of one substep (device memory; read back after the graph)
struct BodyLoop {
  int32_t ite;        // Newton iterations done
  int32_t go;         // 1 while the loop continues
  uint32_t status;    // MGPBD_STATUS_* bits
  int32_t pass;       // CG pass of this Newton iteration
  int32_t cg_total;   // CG iterations of the substep
  int32_t cg_newton;  // CG iterations of this Newton iteration
  int32_t left;       // CG iterations left in this Newton iteration
  int32_t cg_launches;
  int32_t n_log;      // log entries written
  int32_t pad;
  double residual0, residual;  // |b| over all bodies: first, latest
  double omega_min;            // smallest line-search step of the last iteration
  JcgCtl jc;                   // the next CG pass
};

// Per Newton iteration: |b| over the bodies, CG iterations, smallest step
struct BodyLogEntry {
  double r, cg, omega;
};

struct BodyArrays {
  int32_t nb = 0, n_chunks = 0;
  const int32_t* chunk_ptr = nullptr;  // (nb + 1) each body's chunks,
  const int32_t* chunk_idx = nullptr;  // ascending
  const double* partials = nullptr;    // chunk partials, k * n_chunks + c
  int32_t* active = nullptr;           // 1 while the body's loop runs
  double* r0 = nullptr;                // |b_body| at the first iteration
  double* r = nullptr;                 // |b_body|, latest
  double* bnorm = nullptr;             // |b_body| of active bodies, else 0
  double* sq = nullptr;                // scratch: per-body sums
  double* cur = nullptr;               // line search: the current norm^2
  int32_t* newton = nullptr;           // Newton iterations per body
  float* omega = nullptr;              // line-search step per body
  double* omega_h = nullptr;           // the same, as the host keeps it
  BodyLogEntry* log = nullptr;         // log_cap entries (maxiter + 1)
  int32_t log_cap = 0;
};

struct BodyLimits {
  float atol, rtol, tol_cg, rel_tol_cg;
  int32_t maxiter, maxiter_cg;
  int32_t per_body_cg;  // 1: the CG is per body (its own bounds); one pass
};

// Loop state reset for a new substep (all bodies active)
void launch_bodies_reset(const BodyArrays& ba, BodyLoop* L, cudaStream_t s);
// From chunk partials of (C + alpha lambda)^2: per-body |b|, the stopping
// tests, the first CG pass of the iteration; sets the loop's conditional
// (go) through `handle`
void launch_bodies_residual(const BodyArrays& ba, BodyLoop* L, const BodyLimits& lim,
                            cudaGraphConditionalHandle handle, cudaStream_t s);
// After a CG pass (st), from chunk partials of the CG residual squared: the
// per-body check and the next pass (or none)
void launch_bodies_verify(const BodyArrays& ba, BodyLoop* L, const CgState* st,
                          const BodyLimits& lim, cudaStream_t s);
// Per-body sums of the chunk partials into ba.cur (the line search's
// current norm)
void launch_bodies_cur(const BodyArrays& ba, cudaStream_t s);
// From chunk partials of n_trials trial norms: each active body's step,
// its iteration count, the log entry; ite += 1
// warm_substep: at the first Newton iteration, x = the previous substep's
// first solution and the next CG pass starts from it (when *have_prev)
void launch_bodies_warm_in(BodyLoop* L, const int32_t* have_prev, float* x, const float* prev,
                           int32_t n, cudaStream_t s);
// ... and after that iteration's solve (no NaN, no cap), keep it
void launch_bodies_warm_out(const BodyLoop* L, int32_t* have_prev, const float* x, float* prev,
                            int32_t n, cudaStream_t s);
void launch_bodies_omega(const BodyArrays& ba, BodyLoop* L, const BodyLimits& lim, int n_trials,
                         cudaStream_t s);

}  // namespace mgpbd
