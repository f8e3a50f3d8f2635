// Host launchers of the MGPBD device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mgpbd {

// Number of blocks used by the deterministic two-stage float64 reductions
// for a vector of n entries; partial buffers must hold this many doubles.
int reduce_blocks(int64_t n);
constexpr int kReduceThreads = 256;
constexpr int kMaxReduceBlocks = 1216;  // 8 x 152 SMs

// ---- per-vertex / per-tet stages (cons/mgpbd_gpu.py) ---------------------
// ctype (nullable: all MGPBD_CONS_ARAP) selects each constraint's type; a
// length constraint's rest length goes to rest_vol
void launch_rest_shape(const float* x_ref, const int32_t* t_i, const int32_t* ctype, int32_t nt,
                       float mu, float dt, float* dm_inv, float* rest_vol, float* alpha,
                       cudaStream_t s);
void launch_predict(float* x, float* v, float* x_old, float* x_pred, const float* invm,
                    int32_t nv, float dt, const float* g, float damp, int kinematic,
                    cudaStream_t s);
void launch_update_vel(const float* x, const float* x_old, float* v, int32_t nv, float dt,
                       float damp, cudaStream_t s);
void launch_constraints(const float* x, const int32_t* t_i, const int32_t* ctype,
                        const float* dm_inv, const float* rest, int32_t nt, float* C,
                        float* gradC, cudaStream_t s);
// b = -(C + alpha*lambda); partials of |b|^2 (float64)
void launch_rhs(const float* C, const float* alpha, const float* lambda, int32_t nt, float* b,
                double* partials, cudaStream_t s);
// partials of |C + alpha*lambda|^2 (no b written)
void launch_dual_sq(const float* C, const float* alpha, const float* lambda, int32_t nt,
                    double* partials, cudaStream_t s);
// dual residual at x + omega_k * dpos for n_omega step sizes; partials laid
// out [k * blocks + block]
void launch_dual_trial(const float* x, const float* dpos, const double* omegas, int n_omega,
                       const int32_t* t_i, const int32_t* ctype, const float* dm_inv,
                       const float* rest, const float* alpha, const float* lambda, int32_t nt,
                       double* partials, cudaStream_t s);
// lambda += dlam; dpos[v] = sum over incident (t,l) ascending of
// w_v * dlam_t * gradC[t,l] (float32; with dlam_lo, the low part of a
// float-pair dlam, in float64 over dlam + dlam_lo)
void launch_lambda_update(float* lambda, const float* dlam, int32_t nt, cudaStream_t s);
void launch_scatter(const int32_t* inc_ptr, const int32_t* inc_ent, const float* invm,
                    const float* dlam, const float* gradC, float* dpos, int32_t nv, cudaStream_t s,
                    const float* dlam_lo = nullptr);
// per-body reductions of a packed batch over constraint chunks (int2 begin,
// end; each inside one body): partials[c] = sum of (C + alpha lambda)^2
// over chunk c (alpha = null: sum of C^2)
void launch_chunk_dual_sq(const float* C, const float* alpha, const float* lambda,
                          const int32_t* chunks, int32_t n_chunks, double* partials,
                          cudaStream_t s);
// partials[k * n_chunks + c]: chunk c's squared dual residual at x + omega_k dpos
void launch_chunk_trial(const float* x, const float* dpos, const double* omegas, int n_omega,
                        const int32_t* t_i, const int32_t* ctype, const float* dm_inv,
                        const float* rest, const float* alpha, const float* lambda,
                        const int32_t* chunks, int32_t n_chunks, double* partials,
                        cudaStream_t s);
// b_t = 0 where active[cons_body[t]] == 0
void launch_mask_rhs(float* b, const int32_t* cons_body, const int32_t* active, int32_t nt,
                     cudaStream_t s);
// x += omega[vert_body[v]] dpos for free vertices
void launch_apply_bodies(float* x, const float* dpos, const float* invm, const int32_t* vert_body,
                         const float* omega, int32_t nv, cudaStream_t s);
void launch_apply(float* x, const float* dpos, const float* invm, int32_t nv, float omega,
                  cudaStream_t s);

// ---- matrix assembly ------------------------------------------------------
// cons/mgpbd_gpu.py:273-309 on the diagonal-last pattern, plus diag^-1
void launch_fill_A(const int32_t* indptr, const int32_t* indices, const int32_t* t_i,
                   const float* invm, const float* gradC, const float* alpha, int32_t nt,
                   float* data, float* diag_inv, cudaStream_t s);
// cons/mgpcg_gpu.py:183-198 (p = 1 for piecewise-constant P)
void launch_rap_refill(const int32_t* off, const int32_t* idx, const float* fine, int64_t nnz_c,
                       float* coarse, cudaStream_t s);
void launch_diag_inv_pos(const int32_t* diag_pos, const float* data, int32_t n, float* diag_inv,
                         cudaStream_t s);
// cons/sparse_gpu.py:107-121 (linear scan), for caller matrices
void launch_diag_inv_scan(const int32_t* indptr, const int32_t* indices, const float* data,
                          int32_t n, float* diag_inv, cudaStream_t s);

// ---- sparse operators -----------------------------------------------------
struct CsrView {
  int32_t n = 0;
  int64_t nnz = 0;
  const int32_t* indptr = nullptr;
  const int32_t* indices = nullptr;
  const float* data = nullptr;
  const float* diag_inv = nullptr;
  // indices/data are 16-byte aligned and padded by >= 4 elements, so the
  // vectorised row kernel may be used
  bool padded = false;
  // tile shape of the vectorised row kernel (index into the candidate
  // list), -1: chosen from the mean row length
  int shape = -1;
};
// candidate tile shapes of the vectorised row kernel (G lanes x U float4)
constexpr int kNumRowShapes = 8;
// shape index <-> code G * 100 + U (e.g. 406 = 4 lanes x 6 float4)
int row_shape_code(int idx);
int row_shape_index(int code);
// times every candidate shape on `a` (reps Jacobi sweeps y = x + 0.5 D^-1
// (b - A x) each, CUDA events on s, synchronising) and returns the fastest
// shape's index; *best_us gets its time per sweep
int tune_row_shape(const CsrView& a, const float* x, const float* b, float* y, int reps,
                   cudaStream_t s, float* best_us);
// padding (elements) the library allocates after every CSR value/index array
constexpr int64_t kCsrPad = 8;
// y = A x
void launch_spmv(const CsrView& a, const float* x, float* y, cudaStream_t s);
// y = A x and partials of x.y (float64)  -- for CG's p.Ap
void launch_spmv_dot(const CsrView& a, const float* x, float* y, double* partials,
                     cudaStream_t s);
// x_new = x + w * dinv * (b - A x); x == nullptr means x = 0
void launch_jacobi(const CsrView& a, const float* b, const float* x, float* x_new, float w,
                   cudaStream_t s);
// r = b - A x
void launch_residual(const CsrView& a, const float* b, const float* x, float* r, cudaStream_t s);
// bc[I] = sum_{i in I ascending} r[i]  (P^T r with the P^T CSR of members)
void launch_restrict(const int32_t* mem_ptr, const int32_t* mem_rows, const float* r,
                     int32_t n_coarse, float* bc, cudaStream_t s);
// x[i] += xc[agg[i]]
void launch_prolong_add(const int32_t* agg, const float* xc, int32_t n, float* x, cudaStream_t s);

// ---- BLAS-1 (cons/sparse_gpu.py:18-70) ------------------------------------
void launch_dot_partials(const float* a, const float* b, int64_t n, double* partials,
                         cudaStream_t s);
void launch_axpy(float alpha, const float* x, float* y, int64_t n, cudaStream_t s);
void launch_xpay(float alpha, const float* x, float* y, int64_t n, cudaStream_t s);
void launch_scale(float alpha, float* x, int64_t n, cudaStream_t s);
// sums `count` groups of `blocks` partials each into out[g] (float64, fixed order)
void launch_finalize(const double* partials, int blocks, int count, double* out, cudaStream_t s);

// ---- device-driven CG (FAST mode) ----------------------------------------
struct CgState {
  double rz, rz_new, pap, alpha, beta, rr, rr0, tol2;
  int32_t iters, done, status, maxiter;
  int32_t body_runs;  // executions of the captured loop body
  int32_t flags;      // primal warm start: 1 = declined (too stiff to help)
};
// the fused vector kernels read the device state; all return early once done
void launch_cg_init(CgState* st, const double* partials_rz, int blocks, double tol_abs,
                    double tol_rel, int maxiter, cudaStream_t s);
void launch_cg_alpha(CgState* st, const double* partials_pap, int blocks, cudaStream_t s);
// x += alpha p ; r -= alpha Ap ; partials of r.r
void launch_cg_update_xr(const CgState* st, const float* p, const float* ap, float* x, float* r,
                         int64_t n, double* partials, cudaStream_t s);
void launch_cg_check(CgState* st, const double* partials_rr, int blocks, cudaStream_t s);
void launch_cg_beta(CgState* st, const double* partials_rz, int blocks, cudaStream_t s);
// restart from the current iterate: rz from partials, drops status bits
void launch_cg_restart(CgState* st, const double* partials_rz, int blocks, int32_t clear_mask,
                       cudaStream_t s);
// p = z + beta p
void launch_cg_update_p(const CgState* st, const float* z, float* p, int64_t n, cudaStream_t s);

// guarded variants of the V-cycle pieces (no-ops once st->done)
void launch_jacobi_g(const CgState* st, const CsrView& a, const float* b, const float* x,
                     float* x_new, float w, cudaStream_t s);
// same with the weight read from device memory (w_dev) when not null
void launch_jacobi_gw(const CgState* st, const CsrView& a, const float* b, const float* x,
                      float* x_new, float w, const float* w_dev, cudaStream_t s);
void launch_residual_g(const CgState* st, const CsrView& a, const float* b, const float* x,
                       float* r, cudaStream_t s);
void launch_restrict_g(const CgState* st, const int32_t* mem_ptr, const int32_t* mem_rows,
                       const float* r, int32_t n_coarse, float* bc, cudaStream_t s);
void launch_prolong_add_g(const CgState* st, const int32_t* agg, const float* xc, int32_t n,
                          float* x, cudaStream_t s);
void launch_spmv_dot_g(const CgState* st, const CsrView& a, const float* x, float* y,
                       double* partials, cudaStream_t s);
void launch_dot_partials_g(const CgState* st, const float* a, const float* b, int64_t n,
                           double* partials, cudaStream_t s);
// dense float64 Cholesky solve on the coarsest level: x = L^-T L^-1 b
void launch_dense_chol_solve(const CgState* st, const double* L, int32_t n, const float* b,
                             float* x, cudaStream_t s);
// dense factorisation (single block): A (n x n, from CSR) -> L, float64
void launch_dense_chol_factor(const CsrView& a, double* work, int32_t n, int32_t* info,
                              cudaStream_t s);

}  // namespace mgpbd
