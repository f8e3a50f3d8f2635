// Matrix-free application of the MGPBD system matrix A = J W J^T + alpha~
// (the matrix _fill_A_kernel assembles, cons/mgpbd_gpu.py:273-309) and the
// Chebyshev-preconditioned CG built on it (FAST mode).
//
//   A x = J W J^T x + alpha~ x
//   vertex phase:  u_v = w_v * sum_{(t,l): t_i[4t+l] = v} x_t g_{t,l}
//   tet phase:     (A x)_t = sum_l g_{t,l} . u_{t_i[4t+l]} + alpha~_t x_t
//
// Per application this streams the gradients twice (tet-major gradC and a
// vertex-major copy gV with the tet id in .w, 48 + 64 B per tet) instead of
// the 8 B per nonzero of the CSR matrix (~81 nonzeros per row): ~45 MB
// instead of ~214 MB at 320k tets, small enough to stay in the 129 MB L2
// across the thousands of applications of one solve.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "kernels.cuh"

namespace mgpbd {

constexpr int kMaxCheb = 32;
constexpr int kMaxLanczos = 32;

// Chebyshev coefficients (written by the host after each Lanczos estimate)
struct ChebCoef {
  double theta;           // (hi + lo) / 2 of the interval on D^-1 A
  double lmax;            // Lanczos estimate of lambda_max(D^-1 A)
  float c1[kMaxCheb];     // rho_i * rho_{i-1}
  float c2[kMaxCheb];     // 2 rho_i / delta
  float inv_theta;
  int32_t degree;
};

// Device scalars of the Chebyshev-preconditioned CG; lives next to CgState.
struct JState {
  ChebCoef cf;
  double lz_a[kMaxLanczos];  // Lanczos diagonal
  double lz_b[kMaxLanczos];  // Lanczos off-diagonal
  double scale;              // scratch scalar (1/|q| of the start vector)
  uint32_t ticket[4];        // last-block counters of the fused reductions
};

struct JView {
  int32_t nt = 0, nv = 0;
  const int32_t* t_i = nullptr;      // (nt, 4)
  const float* gradC = nullptr;      // (nt, 4, 3)
  const float4* gT = nullptr;        // gradC as 3 planes of nt float4 (persistent CG)
  const float4* gV = nullptr;        // (ne) vertex-major (g, tet id)
  const int32_t* inc_ptr = nullptr;  // (nv + 1)
  int64_t ne = 0;                    // incidence entries (<= 4 nt: repeated slots left out)
  const float* invm = nullptr;       // (nv)
  const float* alpha = nullptr;      // (nt)
  const float* dinv = nullptr;       // (nt) 1 / diag(A)
  bool unit_dinv = false;            // dinv is all ones (unscaled Chebyshev base)
  float4* u = nullptr;               // (nv) vertex scratch
  // compact length constraints (the persistent kernels' unstaged tet
  // phases): constraints n4 .. nt-1 are length constraints whose gradient n
  // is gE[t - n4] and vertices qE[t - n4]; n4 = nt when there are none
  int32_t n4 = 0;
  float4* gE = nullptr;
  const int2* qE = nullptr;
};

// gV[k] = (gradC[inc_ent[k]], tet id) and 1/diag(A) per tet (1 with
// unit_dinv: the unscaled Chebyshev base); with gT, also
// the gradients as three planes (gT[t], gT[nt + t], gT[2 nt + t] = the
// float4s 0, 1, 2 of tet t), so a warp's loads of one float4 per tet are
// contiguous
void launch_jform_prepare(const JView& j, const int32_t* inc_ent, float4* gV, float* dinv,
                          float4* gT, bool unit_dinv, cudaStream_t s);
// y = A x (plain), for tests and the power iteration
void launch_jform_apply(const JView& j, const float* x, float* y, cudaStream_t s);
// `steps` Lanczos steps on S = D^-1/2 A D^-1/2 from a fixed start vector;
// the tridiagonal coefficients land in js->lz_a / js->lz_b (q, qprev, w:
// nt floats of scratch)
void launch_jform_lanczos(const JView& j, float* q, float* qprev, float* w, double* partials,
                          JState* js, int steps, cudaStream_t s);
// On the device, from the `steps` Lanczos coefficients in js: the largest
// eigenvalue of the tridiagonal (bisection), and js->cf = the Chebyshev
// coefficients of `degree` on [1.02 lmax lo_ratio, 1.02 lmax]; a lmax that
// is not finite and positive ORs MGPBD_STATUS_NAN into *status (if given)
// and leaves js->cf.lmax NaN or <= 0 for the host to see.
void launch_cheb_coefficients(JState* js, int steps, int degree, double lo_ratio,
                              uint32_t* status, cudaStream_t s);

// CG with the degree-k Chebyshev preconditioner (k >= 1; k = 1 is scaled
// Jacobi), scalars on the device.  init: x = 0, r = b, z = M^-1 r, p = z.
struct JVecs {
  const float* b = nullptr;
  float* x = nullptr;
  double* xd = nullptr;  // float64 copy of x (accumulated)
  double* r = nullptr;   // float64 residual
  float* z = nullptr;
  float* d = nullptr;
  float* p = nullptr;
  float* ap = nullptr;
  double* partials = nullptr;
};
void launch_jcg_init(const JView& j, const JVecs& v, JState* js, CgState* st, double tol_abs,
                     double tol_rel, int maxiter, cudaStream_t s);
// Chebyshev steps 1..degree-1 of z = M^-1 r (the last one reduces r.z:
// init -> rz, otherwise beta and the iteration count)
void launch_jcg_cheb_steps(const JView& j, const JVecs& v, JState* js, CgState* st, int degree,
                           bool init, cudaStream_t s);
// one CG iteration: p = z + beta p, Ap, alpha, x/r update and convergence
// test, z = M^-1 r, beta (all kernels are no-ops once st->done)
void launch_jcg_body(const JView& j, const JVecs& v, JState* js, CgState* st, int degree,
                     cudaStream_t s);
// Grid barrier state of the persistent CG kernels (zeroed before each launch)
struct GridSync {
  unsigned long long count;  // arrivals; barrier n completes at n * grid
  unsigned int err;          // 1: a block gave up waiting
  unsigned int pad;
};

// float32 work vectors of the persistent CG (all nt long but partials)
struct JcgVecs {
  const float* b = nullptr;
  float* x = nullptr;   // solution (compensated sum during the solve)
  float* xc = nullptr;  // Kahan compensation of x
  float* r = nullptr;
  float* z = nullptr;
  float* d = nullptr;
  float* p = nullptr;
  float* ap = nullptr;
  double* partials = nullptr;
  int64_t partials_capacity = 0;  // doubles; needs 3 * the plan's grid
  GridSync* gs = nullptr;
  float4* ulo = nullptr;  // warm start: nv float4 scratch
};
// Work split of the persistent kernel for one mesh on the current device:
// the cooperative grid, and, when the block data fits in shared memory
// (staged), each block's vertex range (balanced by incident entries) and
// 32-aligned tet range with the largest per-block counts.
struct JcgPlan {
  bool staged = false;
  int grid = 0;   // resident blocks of the cooperative launch
  int smem = 0;   // dynamic shared memory per block (staged)
  int32_t vmax = 0, tmax = 0, emax = 0;
  std::vector<int32_t> vb, tb;  // grid + 1 boundaries each (staged)
};
// allow_staged = false: the unstaged plan (operator read from L2) even when
// the staged one would fit
JcgPlan jcg_plan(const std::vector<int32_t>& inc_ptr, int32_t nv, int32_t nt,
                 bool allow_staged = true);
// The whole CG solve (init, iterations to the tolerance or maxiter, the
// Chebyshev preconditioner of `degree`) as one cooperative kernel; st is
// zeroed and then filled like the per-phase path fills it.  part_dev holds
// plan.vb then plan.tb on the device (staged plans).  warm: start from the
// x on entry (r = b - A x) instead of 0; the tolerance stays relative to
// |b|.  A barrier wait longer than spin_limit_s sets
// MGPBD_STATUS_SYNC_TIMEOUT in st->status.
// With ctl (device memory), a launch captured into a graph takes its
// tolerance, iteration limit and start from there when it runs (tol_abs,
// maxiter and warm are then ignored), or returns at once when ctl->skip is
// set, writing nothing.
struct JcgCtl {
  double tol_abs;
  int32_t maxiter;
  int32_t warm;
  int32_t skip;
  int32_t pad;
};
void launch_jcg_persistent(const JView& j, const JcgVecs& v, const JcgPlan& plan,
                           const int32_t* part_dev, const JState* js, CgState* st, double tol_abs,
                           double tol_rel, int maxiter, int degree, bool warm, double spin_limit_s,
                           cudaStream_t s, const JcgCtl* ctl = nullptr);

// Packed bodies: the per-body CG of launch_jcg_bodies (A block diagonal
// over the bodies).  Device arrays; the chunks and body lists are constant
// per pack, the scalars are the kernel's scratch.
struct BodyCg {
  int32_t nb = 0, nch = 0;
  const int2* ch = nullptr;        // CG chunks (begin, end), each inside one body
  const int32_t* chb = nullptr;    // body of each chunk
  const int32_t* bptr = nullptr;   // per body: its chunks, ascending (nb + 1)
  const int32_t* bidx = nullptr;
  const int32_t* cbody = nullptr;  // body of each constraint
  double* cp = nullptr;            // 3 planes of nch chunk partials
  double* sc = nullptr;            // 5 planes of nb per-body scalars
  float* fa = nullptr;             // per-body alpha
  float* fb = nullptr;             // per-body beta
  int32_t* done = nullptr;         // per body: its CG has stopped
  int32_t* iters = nullptr;        // per body: CG iterations
  uint32_t* ndone = nullptr;       // bodies stopped (zeroed by the launch)
};
// One CG per body in one cooperative launch (unstaged phases, own grid):
// each body's dot products, alpha, beta and stopping test (|r_b| below
// max(tol_abs, tol_rel |b_b|)) are its own; a stopped body keeps x and r.
// st->iters = the iterations of the longest body; status bits as
// launch_jcg_persistent (CG_MAXITER when a body reached maxiter).  ctl as
// there.
void launch_jcg_bodies(const JView& j, const JcgVecs& v, const BodyCg& bc, const JState* js,
                       CgState* st, double tol_abs, double tol_rel, int maxiter, int degree,
                       bool warm, double spin_limit_s, cudaStream_t s,
                       const JcgCtl* ctl = nullptr);

// Work vectors of the primal persistent CG (pcg.cu): vertex vectors are
// float4 per vertex (xyz used), s is per tet.
struct PcgVecs {
  const float* b = nullptr;  // dual right-hand side (nt)
  float* dlam = nullptr;     // dual solution (nt)
  float4 *y = nullptr, *yc = nullptr, *r = nullptr, *z = nullptr, *d = nullptr, *p = nullptr,
         *q = nullptr, *rhs = nullptr, *bi0 = nullptr, *bi1 = nullptr;
  float* s = nullptr;
  double* partials = nullptr;
  int64_t partials_capacity = 0;  // doubles; needs 4 * the plan's grid
  GridSync* gs = nullptr;
};
// Whether a staged plan's shared memory also fits the primal kernel, and
// the primal kernel's cooperative grid when nothing is staged.
bool pcg_plan_fits(JcgPlan& plan);
int pcg_unstaged_grid();
// The dual solve A dlam = b by CG on the primal system K y = J^T alpha~^-1 b
// (one cooperative kernel; see pcg.cu), stopping on the dual residual
// (tol_abs, tol_rel |b|), on maxiter, or, with stall_its > 0, once the dual
// residual has not fallen by 10 % for stall_its iterations.  With max_amp >
// 0 it declines at once (st->flags = 1) when the dual residual of its start
// exceeds max_amp |b|; st->rz_new holds that ratio.  st is zeroed and then
// filled like the dual path fills it (iters = primal iterations).
void launch_pcg_primal(const JView& j, const PcgVecs& v, const JcgPlan& plan,
                       const int32_t* part_dev, CgState* st, double tol_abs, double tol_rel,
                       int maxiter, int degree, float cheb_lo, int stall_its, double max_amp,
                       double spin_limit_s, cudaStream_t s);

// deterministic start vector of the power iteration
void launch_seed(float* v, int32_t n, cudaStream_t s);
// x (float32 output) = xd
void launch_jcg_finish(const JVecs& v, int32_t nt, const CgState* st, cudaStream_t s);

}  // namespace mgpbd
