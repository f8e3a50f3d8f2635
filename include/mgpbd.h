/*
 * mgpbd.h - C ABI of libmgpbd.so, a GB300 (sm_103a) implementation of the
 * MGPBD global XPBD step of JamesYang-7/Controllable_PBD_3D.
 *
 * The reference exposes this step as the Python class `MGPBDSolverGPU`
 * (cons/mgpbd_gpu.py:20-446) backed by `GPUMultigridSolver`
 * (cons/mgpcg_gpu.py:17-329), `GPUSparseMatrix` and free BLAS-1 kernels
 * (cons/sparse_gpu.py:18-144) and the host hierarchy builder
 * (cons/tet_aggregation.py:11-211).  Each entry point below names the
 * reference symbol it replaces.
 *
 * Conventions
 *  - Every function returns 0 on success or a negative MGPBD_E* code;
 *    mgpbd_strerror() turns it into text.  Nothing throws across the ABI.
 *  - Array arguments documented as "device" are CUDA device pointers owned
 *    by the caller; they must stay valid while the handle uses them.  Arrays
 *    documented as "host" are ordinary host memory.
 *  - A handle is used from one host thread at a time and issues its work on
 *    the stream given to mgpbd_set_stream (default: the legacy stream).
 *    Separate handles are independent.
 *  - Layouts follow the reference's Taichi fields: positions (NV,3) float32,
 *    flat tet indices t_i (4*NT) int32, per-tet gradients (NT,4,3) float32,
 *    CSR matrices as (indptr int32[n+1], indices int32[nnz], data float32[nnz]).
 */
#ifndef MGPBD_H_
#define MGPBD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes -------------------------------------------------------- */
#define MGPBD_OK 0
#define MGPBD_EINVAL -1      /* bad argument (null pointer, size, order)      */
#define MGPBD_ECUDA -2       /* a CUDA runtime call failed                    */
#define MGPBD_ENOMEM -3      /* device or host allocation failed              */
#define MGPBD_ESTATE -4      /* call out of order (e.g. step before init)     */
#define MGPBD_ENUMERIC -5    /* NaN/Inf met in the solve (status word set)    */
#define MGPBD_ERANGE -6      /* size beyond an index-type or table limit      */
#define MGPBD_ENOTSUP -7     /* option not supported by this build            */

/* ---- device status word bits (mgpbd_get_status) ------------------------- */
#define MGPBD_STATUS_NAN 1u          /* non-finite residual / scalar seen      */
#define MGPBD_STATUS_PAP_NONPOS 2u   /* CG curvature p.Ap <= 0                 */
#define MGPBD_STATUS_CG_MAXITER 4u   /* a CG solve hit maxiter_cg              */
#define MGPBD_STATUS_NEWTON_MAXITER 8u /* the Newton loop hit maxiter          */
#define MGPBD_STATUS_STALL 16u       /* CG residual stopped decreasing         */
#define MGPBD_STATUS_SYNC_TIMEOUT 32u /* a grid barrier wait of the persistent
                                        CG kernel gave up (solve failed)      */

/* ---- solver options ------------------------------------------------------ */
/* Algorithm variants.  PARITY reproduces the reference step
 * (cons/mgpbd_gpu.py:397-446 with cons/mgpcg_gpu.py:214-329): weighted
 * Jacobi smoothing with omega_jacobi, min(50, n) Jacobi sweeps on the
 * coarsest level, absolute CG tolerance tol_cg, host-checked loops.
 * FAST keeps the same Newton/PCG structure but runs every loop on the device
 * (scalars never leave the GPU inside a CG solve), smooths with a weight set
 * from an estimate of lambda_max(D^-1 A) so the smoother cannot diverge on
 * stiff material, solves the coarsest level densely in float64 and stops CG
 * on the relative residual rel_tol_cg as well as tol_cg. */
#define MGPBD_MODE_PARITY 0
#define MGPBD_MODE_FAST 1

#define MGPBD_COARSE_JACOBI 0    /* min(50,n) weighted Jacobi sweeps (ref)    */
#define MGPBD_COARSE_DENSE_F64 1 /* float64 Cholesky of the coarsest matrix   */

#define MGPBD_SMOOTH_JACOBI 0    /* x += w D^-1 (b - A x), w = omega_jacobi   */
#define MGPBD_SMOOTH_JACOBI_SAFE 1 /* same, w = min(omega, 4/(3 lmax)) per level */

typedef struct mgpbd_params {
  /* reference constructor arguments (cons/mgpbd_gpu.py:22-42) */
  float dt;
  float mu;
  float damp;
  float gravity[3];
  int32_t maxiter;
  float atol;
  float rtol;
  int32_t maxiter_cg;
  float tol_cg;
  int32_t n_smooth;
  float omega_jacobi;
  int32_t setup_interval; /* accepted, unused (as in the reference GPU path) */
  int32_t use_line_search;
  /* extensions (defaults from mgpbd_default_params reproduce the reference) */
  int32_t mode;           /* MGPBD_MODE_*                                     */
  float rel_tol_cg;       /* 0: absolute tol_cg only (reference)              */
  int32_t coarse_solver;  /* MGPBD_COARSE_*                                   */
  int32_t smoother;       /* MGPBD_SMOOTH_*                                   */
  int32_t max_levels;     /* extra levels by matrix-graph aggregation (0=ref) */
  int32_t max_coarse;     /* coarsest-level target size (reference: 400)      */
  int32_t kinematic_pins; /* 1: invm==0 vertices skip the prediction          */
  int32_t coarse_sweeps;  /* coarsest Jacobi sweeps, 0 = min(50,n) (ref)      */
  /* 1: reproduce the reference PCG as shipped, where vcycle(0) writes its
   * residual into the CG residual vector (cons/mgpcg_gpu.py:239-240 share
   * self._r[0] with :275,303); 0 (default): the V-cycle has its own. */
  int32_t cg_alias;
  /* > 0: alpha~ = compliance / dt^2 for every tet (the XPBD convention of
   * cons/length.py:30) instead of 1 / (mu dt^2 V_t) (cons/mgpbd_gpu.py:151) */
  float compliance;
  /* CG preconditioner: MGPBD_PRECOND_VCYCLE (the reference's aggregation
   * V-cycle on CSR matrices) or MGPBD_PRECOND_CHEB (FAST mode only: a
   * degree-`cheb_degree` Chebyshev polynomial in D^-1 A on the interval
   * [lambda_max * cheb_lo, lambda_max], with A applied matrix-free from the
   * constraint gradients; no CSR assembly per Newton iteration) */
  int32_t precond;
  int32_t cheb_degree;
  float cheb_lo;
  /* FAST mode: 1 (default) runs each CG solve as one CUDA graph with a
   * device-side while loop; 0 launches the same kernels from a host loop
   * that checks the device state every 8 iterations (for profilers that
   * cannot look inside conditional graphs).  With packed bodies
   * (mgpbd_set_bodies), 1 runs each whole substep's Newton loop as one
   * captured graph (decisions taken on the device; captured at the first
   * solve and again when the barrier limit changes), 0 drives the same
   * kernels from the host loop; both give the same results bit for bit. */
  int32_t use_graph;
  /* FAST mode with MGPBD_PRECOND_CHEB: 1 (default) runs each CG solve as ONE
   * cooperative persistent kernel (grid barriers between its phases, float32
   * vectors, compensated solution sum); 2 the same without staging the
   * operator in shared memory (read from L2, as for meshes too large to
   * stage); 0 runs the per-phase kernels (use_graph selects graph or host
   * loop for those). */
  int32_t persistent;
  /* FAST mode, MGPBD_PRECOND_CHEB, persistent: 1 warm-starts each solve
   * through the primal system K y = J^T alpha~^-1 b with K = W^-1 +
   * J^T alpha~^-1 J on the free vertices, dlam = alpha~^-1 (b - J y)
   * (Woodbury identity; block-Jacobi Chebyshev preconditioner), run until
   * the dual residual |b - A dlam| falls below primal_tol |b| or stalls;
   * CG on A then continues from that dlam to the usual tolerance.  The
   * primal start dlam = alpha~^-1 b can have a dual residual far above |b|
   * (by the stiffness ratio), so in float32 the primal CG alone cannot
   * always reach 1e-6; it does the coarse part of the work at about half
   * the cost per unit of residual reduction.  The warm start is declined
   * (CG on A from 0) when that ratio exceeds 1e6: beyond it the hand-over
   * loses accuracy the float32 dual CG does not win back.  0 (default):
   * CG on A only. */
  int32_t primal;
  float primal_tol;  /* relative dual residual of the hand-over (1e-2)     */
  /* MGPBD_PRECOND_LEARNED: the judged first V-cycle of a solve keeps the
   * network iff E_net <= learned_accept * E_plain, E = 1/2 e^T A_c e -
   * e^T r_c of the two coarse corrections (both negative when they help):
   * 0.1 (default) keeps a network that achieves at least a tenth of the
   * coarse-energy decrease of the reference's sweeps (the coarse level is
   * a small part of this system's convergence, so the test only has to
   * catch a network that does not correct at all); 1 demands as much. */
  float learned_accept;
  /* MGPBD_PRECOND_LEARNED: a solve whose CG residual makes no new minimum
   * for this many iterations (default 1000) falls back to the plain
   * V-cycle (restarting CG from its iterate); 0 disables the test (p.Ap <= 0
   * and NaN still fall back).  CG residual norms plateau for a few hundred
   * iterations in ordinary solves of stiff bodies. */
  int32_t learned_stall;
  /* MGPBD_PRECOND_CHEB: the base the Chebyshev polynomial is built on.
   * MGPBD_CHEB_JACOBI (0, default): a polynomial in D^-1 A, D = diag(A).
   * MGPBD_CHEB_UNSCALED (1): a polynomial in A itself.  With one compliance
   * for every constraint, the null space of J^T (most of constraint space
   * when constraints outnumber vertex coordinates) is the single eigenvalue
   * alpha~ of A; Jacobi scaling spreads it over alpha~ / d_i, and with
   * gradients of very different sizes (volume vs length constraints) that
   * band sits at the bottom of the spectrum, where CG pays for it.  No
   * counterpart in the reference. */
  int32_t cheb_scale;
  /* Packed bodies (mgpbd_set_bodies): 1 (default) solves each Newton system
   * with one CG per body in one persistent launch (each body's dot
   * products, alpha, beta and stopping test its own, |r_b| below
   * max(tol_cg, rel_tol_cg |b_b|)); 0 runs one CG over the whole pack to
   * rel_tol_cg of the pack's |b| and then checks each body, continuing from
   * the iterate while some body misses its bound.  No counterpart in the
   * reference (one body per solver). */
  int32_t body_cg;
  /* FAST mode, MGPBD_PRECOND_CHEB, persistent, dual (primal 0), one body:
   * 1 starts the first Newton iteration's CG of each substep from the
   * previous substep's first solution (its residual b - A x formed in
   * float64) instead of 0; the stopping test is unchanged (relative to
   * |b|).  0 (default): from 0, as the reference (cons/mgpcg_gpu.py:272). */
  int32_t warm_substep;
} mgpbd_params;

#define MGPBD_CHEB_JACOBI 0
#define MGPBD_CHEB_UNSCALED 1

#define MGPBD_PRECOND_VCYCLE 0
#define MGPBD_PRECOND_CHEB 1
/* The V-cycle with its coarse correction (the recursion below level 0,
 * min(50, n) Jacobi sweeps on the reference's two-level hierarchy,
 * cons/mgpcg_gpu.py:216-224) replaced by the learned linear correction
 * e_c = w * r_c / diag(A_c), w from a trained network on the
 * level-1 graph (mgpbd_net_*, attached with mgpbd_set_coarse_net), computed
 * once per solve (a fixed linear preconditioner, so standard CG applies),
 * host-checked every iteration.  The plain
 * V-cycle stays as judge and fallback: the first V-cycle of every solve
 * computes both coarse corrections and keeps the network only if its
 * coarse energy 1/2 e^T A_c e - e^T r_c (lower = closer to A_c^-1 r_c in
 * the energy norm) passes the test set by learned_accept; a solve whose
 * residual makes no new minimum for learned_stall iterations (or meets
 * p.Ap <= 0 / NaN) falls back to the plain V-cycle, restarting CG from its
 * current iterate. */
#define MGPBD_PRECOND_LEARNED 2

typedef struct mgpbd_stats {
  int32_t newton_iters;     /* Newton iterations run in the last solve        */
  int32_t cg_iters_total;   /* CG iterations summed over those                */
  int32_t cg_iters_last;    /* CG iterations of the last Newton iteration     */
  int32_t n_levels;         /* multigrid levels                               */
  double residual0;         /* dual residual norm at Newton iteration 0       */
  double residual;          /* dual residual norm at the last check           */
  double omega_last;        /* last line-search step                          */
  uint32_t status;          /* MGPBD_STATUS_* bits of the last solve          */
  int64_t nnz[8];           /* nonzeros per level                             */
  int64_t rows[8];          /* rows per level                                 */
  int32_t cg_path;          /* MGPBD_CGPATH_* the CG solves run on            */
  int32_t cg_grid;          /* blocks of the persistent kernel (0 otherwise)  */
  int32_t cg_iters_warm;    /* of cg_iters_total: primal warm-start iterations */
  int32_t cg_launches;      /* persistent kernel launches in the last solve   */
  double ms_warm;           /* GPU time of the primal warm-start kernels and  */
  double ms_dual;           /* of the dual persistent kernels, last solve     */
  double warm_amp;          /* dual residual / |b| of the primal start (last) */
  int32_t warm_declined;    /* Newton iterations whose warm start declined    */
  /* MGPBD_PRECOND_LEARNED, last solve: */
  int32_t learned_fallbacks; /* solves that fell back to the plain V-cycle     */
  int32_t learned_rejected;  /* solves whose first coarse correction the plain
                                V-cycle judged better (network not used)      */
  int32_t learned_solves;    /* solves that kept the network to the end       */
  double coarse_energy_learned; /* coarse energies of the judged first        */
  double coarse_energy_plain;   /* V-cycle, summed over the solves            */
} mgpbd_stats;

#define MGPBD_CGPATH_KERNELS 0      /* one kernel (or graph node) per operation */
#define MGPBD_CGPATH_PERSISTENT 1   /* one cooperative kernel per solve, the
                                       operator read from L2                   */
#define MGPBD_CGPATH_STAGED 2       /* the same with each block's operator data
                                       staged in shared memory                 */
#define MGPBD_CGPATH_PRIMAL 3       /* primal system, one cooperative kernel    */
#define MGPBD_CGPATH_PRIMAL_STAGED 4 /* the same, operator data staged         */

typedef struct mgpbd_solver* mgpbd_handle;

/* Fill *p with the reference's defaults (cons/mgpbd_gpu.py:30-41):
 * mu 1e6, damp 1, maxiter 20, atol 1e-4, rtol 1e-2, maxiter_cg 100,
 * tol_cg 1e-5, n_smooth 2, omega 2/3, setup_interval 10000, line search on,
 * PARITY mode; dt and gravity are zeroed and must be set by the caller. */
void mgpbd_default_params(mgpbd_params* p);

const char* mgpbd_strerror(int code);
/* Text of the last error raised on the calling thread (empty if none). */
const char* mgpbd_last_error(void);
const char* mgpbd_version(void);
/* Number of CUDA kernels this library has launched in the process so far
 * (kernels inside its CUDA graphs are counted each time they run). */
int64_t mgpbd_launch_count(void);

/* Replaces MGPBDSolverGPU.__init__ (cons/mgpbd_gpu.py:22-90). */
int mgpbd_create(const mgpbd_params* params, mgpbd_handle* out);
void mgpbd_destroy(mgpbd_handle h);
/* cudaStream_t passed as void* so the header needs no CUDA include. */
int mgpbd_set_stream(mgpbd_handle h, void* stream);

/* Bind the caller's mesh (device): rest positions x_ref (nv,3), inverse
 * masses invm (nv), tet indices t_i (4*nt), and the state arrays the step
 * mutates: positions x (nv,3) and velocities v (nv,3).  Replaces the
 * constructor's field arguments (cons/mgpbd_gpu.py:22-28,43-49). */
int mgpbd_set_mesh(mgpbd_handle h, const float* x_ref, const float* invm,
                   const int32_t* t_i, int32_t nv, int32_t nt, float* x,
                   float* v);

/* Optional, between mgpbd_set_mesh and mgpbd_init: the aggregation
 * hierarchy to use instead of the built-in tet aggregation
 * (cons/tet_aggregation.py:145-211 / GPUMultigridSolver.setup's Ps,
 * cons/mgpcg_gpu.py:30-173).  Host arrays: level_sizes[n_levels] with
 * level_sizes[0] = nt; agg_ids holds, level after level, level_sizes[l]
 * aggregate ids in [0, level_sizes[l+1]) (every id used).  2 <= n_levels
 * <= 8.  mgpbd_set_mesh clears it. */
int mgpbd_set_hierarchy(mgpbd_handle h, const int32_t* agg_ids, int32_t n_levels,
                        const int32_t* level_sizes);

/* Replaces GPUMultigridSolver.setup (cons/mgpcg_gpu.py:30-173) for a
 * caller's own level-0 matrix instead of a mesh: host CSR arrays (n rows,
 * nnz entries, every row with its diagonal; the caller's column order is
 * kept).  Then, optionally, mgpbd_set_hierarchy (the Ps of setup as
 * aggregate ids: one 1 per row of each P) and mgpbd_init, which builds
 * the Galerkin coarse levels; mgpbd_pcg / mgpbd_vcycle solve with it.  The
 * handle has no mesh (mesh stages return MGPBD_ESTATE); the parameters
 * must select the V-cycle (precond MGPBD_PRECOND_VCYCLE). */
int mgpbd_set_matrix(mgpbd_handle h, int32_t n, int64_t nnz, const int32_t* indptr,
                     const int32_t* indices, const float* data);
/* Replaces update_fine_matrix_data + update_all_coarse_matrices
 * (cons/mgpcg_gpu.py:175-212) of a mgpbd_set_matrix handle: new level-0
 * values (device pointer, nnz, same pattern), 1/diag, coarse refill. */
int mgpbd_update_matrix(mgpbd_handle h, const float* data);

/* Constraint types.  The reference's step has one ARAP constraint per tet
 * (C = |S - I|_F, cons/mgpbd_gpu.py:226-247).  The library also takes, per
 * constraint, the two blocks of a length + volume discretisation:
 *   MGPBD_CONS_LENGTH: C = |x_a - x_b| - L0 (cons/length.py:65-90); the
 *     constraint lists its edge twice in t_i, (a, b, a, b);
 *   MGPBD_CONS_VOLUME: C = det F - 1, F = D_s Dm^-1 (the hydrostatic
 *     constraint of cons/deform3d.py:81-83) on a tet's four vertices.
 * Every constraint keeps 4 slots in t_i, so the assembly, the multigrid
 * hierarchy, the CG kernels and the scatter are shared (a repeated vertex
 * carries a zero gradient).  Length and volume constraints take
 * alpha~ = compliance / dt^2 (compliance > 0 required); a length
 * constraint's rest length is reported in MGPBD_FIELD_REST_VOL. */
#define MGPBD_CONS_ARAP 0
#define MGPBD_CONS_LENGTH 1
#define MGPBD_CONS_VOLUME 2
/* Between mgpbd_set_mesh and mgpbd_init: types (host array of nt
 * MGPBD_CONS_* values), or NULL for all ARAP.  mgpbd_set_mesh clears it;
 * mgpbd_init validates it.  No counterpart in the reference. */
int mgpbd_set_constraint_types(mgpbd_handle h, const int32_t* types);

/* Independent bodies packed into one mesh (vertex ids shifted per body, so
 * A is block diagonal), each with its own Newton loop: per body the
 * residual norm, the stopping test (atol / rtol of its own first residual)
 * and the line-search step of cons/mgpbd_gpu.py:379-446, over one shared
 * block-diagonal CG solve per Newton iteration that is verified per body
 * (each active body's residual <= rel_tol_cg times its right-hand side; CG
 * continues from its iterate while one is not).  A body whose test holds
 * keeps its positions while the others go on.  Host arrays, between
 * mgpbd_set_mesh (or mgpbd_set_constraint_types) and mgpbd_init:
 * vert_off[n_bodies + 1] (body b owns vertices vert_off[b] ..
 * vert_off[b+1]-1, from 0 to nv); segs[3 * n_segs]: constraint ranges
 * (begin, end, body) covering [0, nt) in order.  A constraint may only
 * touch its body's vertices (checked at init).  FAST mode with the
 * persistent Chebyshev CG only.  n_bodies = 0 returns to one Newton loop.
 * No counterpart in the reference. */
int mgpbd_set_bodies(mgpbd_handle h, int32_t n_bodies, const int32_t* vert_off, int32_t n_segs,
                     const int32_t* segs);
/* Per body (n = n_bodies entries each, NULL to skip): Newton iterations,
 * first and last residual norm, last line-search step of the last solve. */
int mgpbd_body_stats(mgpbd_handle h, int32_t n, int32_t* newton_iters, double* residual0,
                     double* residual, double* omega);

/* Wait limit, in seconds [0, 60], of every grid-barrier wait of the
 * persistent CG kernels (default 4).  A wait that reaches it ends the
 * kernel on every block, marks MGPBD_STATUS_SYNC_TIMEOUT and makes the call
 * return MGPBD_ECUDA; the next launch starts afresh, so the handle stays
 * usable.  0 gives up at the first wait that finds another block not yet
 * arrived, which makes a solve fail this way on purpose (how the tests
 * exercise the path).  No counterpart in the reference. */
int mgpbd_set_barrier_limit(mgpbd_handle h, double seconds);

/* Replaces MGPBDSolverGPU.init (cons/mgpbd_gpu.py:92-114): rest shape,
 * sparsity pattern, first A, tet hierarchy, multigrid setup. */
int mgpbd_init(mgpbd_handle h);

/* Replaces MGPBDSolverGPU.step / make_prediction / solve / update_vel
 * (cons/mgpbd_gpu.py:200-219,397-446). */
int mgpbd_step(mgpbd_handle h, int32_t frame);
int mgpbd_make_prediction(mgpbd_handle h);
int mgpbd_solve(mgpbd_handle h, int32_t frame);
int mgpbd_update_vel(mgpbd_handle h);

int mgpbd_get_stats(mgpbd_handle h, mgpbd_stats* out);
/* Block until the handle's stream has finished its queued work. */
int mgpbd_synchronize(mgpbd_handle h);
/* Per-Newton-iteration record of the last solve, the values the reference
 * passes to benchmark.record_iteration (cons/mgpbd_gpu.py:415-416,442-443):
 * rows of 5 doubles (iteration, residual, cg_iters, omega, host seconds on
 * a monotonic clock).  Writes min(max_rows, *n_rows) rows; *n_rows gets the
 * total. */
int mgpbd_newton_log(mgpbd_handle h, int32_t max_rows, double* rows, int32_t* n_rows);
/* Status bits of the last solve (0 = clean). */
int mgpbd_get_status(mgpbd_handle h, uint32_t* status);

/* Device pointer and element count of a solver-owned field, so a caller can
 * read or (for alpha_tilde, lambda) modify it in place.  Field ids: */
#define MGPBD_FIELD_LAMBDA 0      /* (nt)      lambdaf                         */
#define MGPBD_FIELD_CONSTRAINTS 1 /* (nt)      constraints                     */
#define MGPBD_FIELD_GRADC 2       /* (nt,4,3)  gradC                           */
#define MGPBD_FIELD_ALPHA_TILDE 3 /* (nt)      alpha_tilde                     */
#define MGPBD_FIELD_REST_VOL 4    /* (nt)      rest_vol                        */
#define MGPBD_FIELD_DM_INV 5      /* (nt,3,3)  Dm_inv                          */
#define MGPBD_FIELD_X_OLD 6       /* (nv,3)    v_p_old                         */
#define MGPBD_FIELD_X_PREDICT 7   /* (nv,3)    v_predict                       */
#define MGPBD_FIELD_DPOS 8        /* (nv,3)    dpos                            */
#define MGPBD_FIELD_RHS 9         /* (nt)      _b_gpu                          */
#define MGPBD_FIELD_DLAMBDA 10    /* (nt)      _dlam_gpu                       */
#define MGPBD_FIELD_A_DATA 11     /* (nnz0)    level-0 matrix values           */
int mgpbd_field(mgpbd_handle h, int32_t field, void** dev_ptr, int64_t* count);

/* CSR arrays of multigrid level `level` (device pointers, library-owned).
 * Level 0 keeps the reference's pattern: per row the sorted neighbours,
 * then the diagonal last (cons/mgpbd_gpu.py:153-194). */
int mgpbd_level_csr(mgpbd_handle h, int32_t level, int32_t* n_rows, int64_t* nnz,
                    int32_t** indptr, int32_t** indices, float** data,
                    float** diag_inv);
/* Number of multigrid levels after mgpbd_init. */
int mgpbd_level_count(mgpbd_handle h, int32_t* n_levels);
/* Aggregate id of each row of `level` (device, length n_rows(level)). */
int mgpbd_level_agg(mgpbd_handle h, int32_t level, int32_t** agg_ids);

/* ---- learned coarse correction (no counterpart in the reference) ---------
 * The reference's V-cycle corrects with min(50, n) Jacobi sweeps on its
 * coarsest level (cons/mgpcg_gpu.py:216-224).  The learned correction is
 * linear in the residual: e_c = w * r_c / diag(A_c), with one weight per
 * aggregate computed from the level-1 matrix A_c by a 3-layer
 * message-passing network (hidden width 64) over its graph and bounded,
 * w_i = c_i sigmoid(y_i) with c_i = 1.9 / sum_j |Ah_ij| (below
 * 2 / sum_j |Ah_ij| no mode is over-corrected, so the V-cycle stays
 * positive definite; 1 / sum_j |Ah_ij| is the l1-Jacobi weight).  With
 * s_i = (1/A_ii)^1/2 and Ah = S A_c S, the network on a node field r is
 *   sigma = rms(S r), u = S r / sigma, a1 = Ah u
 *   H1 = relu(u w1s + a1 w1n + b1)
 *   H2 = relu([H1, Ah H1] W2 + b2), H3 = relu([H2, Ah H2] W3 + b3)
 *   y = H3 wo + bo, e = sigma S y            (mgpbd_net_forward)
 * and y is taken on the field r = sqrt(diag A_c) (mgpbd_net_weights).
 * Parameters: one float32 vector of MGPBD_NET_PARAMS values laid out
 *   w1s[64] w1n[64] b1[64] | W2[128][64] b2[64] | W3[128][64] b3[64] |
 *   wo[64] bo.
 * The dense layers run on the tensor cores with bf16 weights and
 * activations (float32 accumulation).  Training (the library's own backward
 * kernels and Adam) minimises the scaled coarse energy over a batch of
 * restricted residuals r_s (u_s = S r_s / sigma_s):
 *   MGPBD_NET_LOSS_WEIGHTS: v_s = w * u_s, L = mean_s (1/2 v_s^T Ah v_s -
 *                           v_s^T u_s) / n  (the correction the solver uses)
 *   MGPBD_NET_LOSS_FIELD:   L = mean_s (1/2 y_s^T Ah y_s - y_s^T u_s) / n
 *                           with y_s the network on r_s
 * Both are minimised by e = A_c^-1 r.  A CSR graph passed to these calls is
 * (n, nnz, indptr[n+1], indices[nnz], data[nnz], diag_inv[n]): device
 * arrays, column indices in [0, n), indptr[n] == nnz (not checked on the
 * device). */
#define MGPBD_NET_PARAMS 16769
#define MGPBD_NET_LOSS_WEIGHTS 0
#define MGPBD_NET_LOSS_FIELD 1
typedef struct mgpbd_net* mgpbd_net_handle;
/* Glorot-uniform weights from `seed` (splitmix64), zero biases. */
int mgpbd_net_create(uint64_t seed, mgpbd_net_handle* out);
void mgpbd_net_destroy(mgpbd_net_handle net);
/* Device pointers of the parameter and gradient vectors (MGPBD_NET_PARAMS
 * floats each).  After writing the parameters, call mgpbd_net_sync_params. */
int mgpbd_net_params(mgpbd_net_handle net, float** params, float** grad);
int mgpbd_net_sync_params(mgpbd_net_handle net, void* stream);
/* w = per-aggregate weights of the graph (device vector of n). */
int mgpbd_net_weights(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                      const int32_t* indices, const float* data, const float* diag_inv,
                      float* w, void* stream);
/* e = max(w, 0) * diag_inv * r (device vectors of n; weights from
 * mgpbd_net_weights are already positive). */
int mgpbd_net_apply(int32_t n, const float* w, const float* diag_inv, const float* r, float* e,
                    void* stream);
/* e = the network on the field r (device vectors of n). */
int mgpbd_net_forward(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                      const int32_t* indices, const float* data, const float* diag_inv,
                      const float* r, float* e, void* stream);
/* Loss (MGPBD_NET_LOSS_*) and gradient (into the gradient vector) of the
 * batch of n_samples residuals stored back to back (device, n_samples * n
 * floats); *loss is host memory, the call returns after it is copied back. */
int mgpbd_net_loss_grad(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                        const int32_t* indices, const float* data, const float* diag_inv,
                        const float* samples, int32_t n_samples, int32_t mode, double* loss,
                        void* stream);
/* One bias-corrected Adam step from the gradient vector. */
int mgpbd_net_adam(mgpbd_net_handle net, float lr, float beta1, float beta2, float eps,
                   void* stream);
/* `steps` Adam steps of the MGPBD_NET_LOSS_WEIGHTS loss on batches of
 * `batch` samples taken cyclically from the n_samples residuals (step k
 * uses samples (k*batch + i) mod n_samples); losses (host, `steps` doubles)
 * receives each step's loss; one host sync. */
int mgpbd_net_train(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                    const int32_t* indices, const float* data, const float* diag_inv,
                    const float* samples, int32_t n_samples, int32_t batch, int32_t steps,
                    float lr, double* losses, void* stream);

/* Attach a network (or NULL) for MGPBD_PRECOND_LEARNED; the caller keeps it
 * alive while the solver may use it.  Its coarse graph is level 1. */
int mgpbd_set_coarse_net(mgpbd_handle h, mgpbd_net_handle net);
/* Training data from the plain solver: while capacity > 0, every `every`-th
 * plain V-cycle (counting from this call) stores its restricted level-1
 * residual r_c into rc[k * n1 ...] and the plain coarse correction (the
 * reference's coarsest-level sweeps) into ec[k * n1 ...] (device buffers
 * of capacity * n1 floats, n1 = rows of level 1), k = 0 .. capacity-1.
 * CG solves run from a host loop (not a CUDA graph) while recording.
 * capacity 0 stops; mgpbd_record_count gives the pairs stored. */
int mgpbd_record_coarse(mgpbd_handle h, float* rc, float* ec, int32_t capacity, int32_t every);
int mgpbd_record_count(mgpbd_handle h, int32_t* count);

/* ---- row-kernel autotuner (no counterpart in the reference) ---------------
 * The CSR kernels of the V-cycle (SpMV, Jacobi sweep, residual) process a
 * row with G lanes, each loading U float4 values and int4 columns per pass.
 * The library picks (G, U) from the mean row length; the autotuner times
 * every candidate shape on each multigrid level's own matrix instead.
 * Shapes are named by the code G * 100 + U (e.g. 406).  A shape changes the
 * summation order inside a row, so results can differ in the last bits
 * between shapes; a fixed shape repeats bit for bit. */
/* Candidate codes (codes: room for *count entries; NULL to query *count). */
int mgpbd_row_shapes(int32_t* codes, int32_t* count);
/* After mgpbd_init: time each candidate (reps Jacobi sweeps, CUDA events on
 * the handle's stream, synchronising) on every level and keep the fastest;
 * codes[l] and us_per_sweep[l] (host, n_levels entries, either may be NULL)
 * receive the choice and its time per sweep.  Values of the level vectors
 * are overwritten. */
int mgpbd_autotune_rows(mgpbd_handle h, int32_t reps, int32_t* codes, float* us_per_sweep);
/* Current shape code of a level (0: chosen from the mean row length), or set
 * one (a code from mgpbd_row_shapes, or 0), e.g. from a cached tuning. */
int mgpbd_level_row_shape(mgpbd_handle h, int32_t level, int32_t* code);
int mgpbd_set_level_row_shape(mgpbd_handle h, int32_t level, int32_t code);

/* ---- per-stage calls (the reference's separately callable kernels) ------ */
/* _compute_C_and_gradC (cons/mgpbd_gpu.py:225-247) at the bound positions */
int mgpbd_compute_constraints(mgpbd_handle h);
/* _fill_A_and_update_gpu (cons/mgpbd_gpu.py:320-324): A values, diag^-1,
 * coarse values by the contribution map (cons/mgpcg_gpu.py:175-212) */
int mgpbd_fill_matrices(mgpbd_handle h);
/* GPUMultigridSolver.update_all_coarse_matrices (cons/mgpcg_gpu.py:200-212)
 * from the current level-0 values (after a caller changed them) */
int mgpbd_refill_coarse(mgpbd_handle h);
/* _compute_rhs_gpu + _residual_norm_gpu (cons/mgpbd_gpu.py:253-267) */
int mgpbd_compute_rhs(mgpbd_handle h, double* residual_norm);
/* GPUMultigridSolver.solve (cons/mgpcg_gpu.py:261-329): solves A x = b on
 * level 0 for device vectors b, x (nt); returns the CG iteration count. */
int mgpbd_pcg(mgpbd_handle h, const float* b, float* x, int32_t* cg_iters);
/* GPUMultigridSolver.vcycle(0) (cons/mgpcg_gpu.py:214-259): z = M^-1 r */
int mgpbd_vcycle(mgpbd_handle h, const float* r, float* z);
/* _zero_dpos + _scatter_dlam_gpu (cons/mgpbd_gpu.py:330-355) for dlam */
int mgpbd_scatter(mgpbd_handle h, const float* dlam);
/* _line_search (cons/mgpbd_gpu.py:379-391); returns omega */
int mgpbd_line_search(mgpbd_handle h, double* omega);
/* _apply_dpos (cons/mgpbd_gpu.py:345-349) */
int mgpbd_apply_dpos(mgpbd_handle h, double omega);

/* y = A x for the level-0 system of the last fill (device vectors, nt):
 * matrix_free = 1 applies J W J^T + alpha~ from the current gradients
 * (the operator _fill_A_kernel assembles, cons/mgpbd_gpu.py:273-309);
 * matrix_free = 2 does the same reusing the vertex-major gradients of the
 * previous call; matrix_free = 0 multiplies by the assembled CSR values. */
int mgpbd_apply_matrix(mgpbd_handle h, int32_t matrix_free, const float* x, float* y);
/* ---- adaptive zones (cons/adaptive_zone.py:14-91) --------------------------
 * `active` is a caller-owned device array of nt int32 (0 passive, 1 active),
 * the reference's AdaptiveZone.tet_active. */
/* AdaptiveZone.update_by_proximity (:40-55): active iff a vertex of the tet
 * (current positions) lies strictly within `radius` of (cx, cy, cz). */
int mgpbd_zone_proximity(mgpbd_handle h, int32_t* active, float cx, float cy, float cz,
                         float radius);
/* AdaptiveZone.update_by_strain (:57-72): active iff the fastest vertex of
 * the tet moved faster than `threshold`, speed = |x - x_old| / dt; x_old is
 * a device (nv, 3) array, or NULL for the solver's v_p_old. */
int mgpbd_zone_strain(mgpbd_handle h, int32_t* active, const float* x_old, float threshold,
                      float dt);
/* AdaptiveZone.expand_zone (:74-85): n_rings rings of growth across faces
 * shared by exactly two tets (the adjacency of cons/tet_aggregation.py:11-37,
 * built on the first call). */
int mgpbd_zone_expand(mgpbd_handle h, int32_t* active, int32_t n_rings);
/* MGPBDAdaptiveSolver._apply_active_mask / _restore_mask
 * (cons/mgpbd_adaptive.py:66-93): saved_alpha (device, nt float) receives
 * alpha~; passive tets get alpha~ = 1e20 (no force); restore copies it back. */
int mgpbd_mask_alpha(mgpbd_handle h, const int32_t* active, float* saved_alpha);
int mgpbd_restore_alpha(mgpbd_handle h, const float* saved_alpha);
/* Host: the face adjacency above as CSR (rows ascending); indptr nt + 1,
 * indices *nnz (pass NULL arrays to query nnz first). */
int mgpbd_host_face_adjacency(const int32_t* t_i, int32_t nt, int64_t* nnz, int32_t* indptr,
                              int32_t* indices);

/* One pass of the library's vectorised CSR row kernel on multigrid level
 * `level`: op 0 y = A x (GPUSparseMatrix.spmv, cons/sparse_gpu.py:123-132),
 * op 1 y = x + omega D^-1 (b - A x) (jacobi_smooth, :134-144). */
int mgpbd_level_sweep(mgpbd_handle h, int32_t level, int32_t op, const float* x,
                      const float* b, float* y, float omega);

/* ---- standalone sparse kernels on caller CSR (device arrays) ------------ */
/* GPUSparseMatrix.spmv (cons/sparse_gpu.py:123-132): y = A x */
int mgpbd_csr_spmv(int32_t n_rows, const int32_t* indptr, const int32_t* indices,
                   const float* data, const float* x, float* y, void* stream);
/* GPUSparseMatrix.jacobi_smooth (cons/sparse_gpu.py:134-144):
 * x_new = x + omega * diag_inv * (b - A x) */
int mgpbd_csr_jacobi(int32_t n_rows, const int32_t* indptr, const int32_t* indices,
                     const float* data, const float* diag_inv, const float* b,
                     const float* x, float* x_new, float omega, void* stream);
/* GPUSparseMatrix.cache_diag_inv (cons/sparse_gpu.py:107-121) */
int mgpbd_csr_diag_inv(int32_t n_rows, const int32_t* indptr, const int32_t* indices,
                       const float* data, float* diag_inv, void* stream);
/* gpu_dot (cons/sparse_gpu.py:18-23); float64 accumulation, fixed order */
int mgpbd_dot(int32_t n, const float* a, const float* b, double* out, void* stream);
/* Same result as mgpbd_dot (within float64 rounding), for callers that may
 * not allocate GPU memory: no counterpart in the reference.  Hosts that own
 * the device memory budget (an engine or tool embedding this library, a
 * real-time loop with a fixed memory plan) can forbid cudaMalloc/cudaFree,
 * which may wait for the whole device and bypass the host's allocator.
 * This entry point allocates nothing: its scratch is a 512 KiB device
 * array inside libmgpbd.so (one float64 per 1024 elements plus the
 * result), held by every GPU that loads the library until the process
 * exits.  n is limited to 67,108,864 elements (MGPBD_ERANGE beyond).  The
 * first call on each device looks up the array's address (with that
 * device current).  All calls share the one array: calls that overlap on
 * the GPU (other streams, other host threads) race and must be serialised
 * by the caller.  `out` is host memory: the call synchronises `stream` and
 * blocks the host until the result is copied back, so it cannot be called
 * while `stream` is being captured into a CUDA graph.  A failure records
 * its message for mgpbd_last_error(). */
int mgpbd_dot_noalloc(int32_t n, const float* a, const float* b, double* out, void* stream);
/* gpu_axpy (:26-30) y += alpha x ; gpu_xpay (:33-37) y = x + alpha y */
int mgpbd_axpy(int32_t n, float alpha, const float* x, float* y, void* stream);
int mgpbd_xpay(int32_t n, float alpha, const float* x, float* y, void* stream);
/* gpu_scale (cons/sparse_gpu.py:52-55) x *= alpha */
int mgpbd_scale(int32_t n, float alpha, float* x, void* stream);

/* ---- host-side structure builders (host arrays, no GPU needed) ---------- */
/* _build_sparsity_pattern (cons/mgpbd_gpu.py:153-194).  Call with indptr ==
 * NULL to get *nnz, then again with indptr (nt+1) and indices (*nnz). */
int mgpbd_host_pattern(const int32_t* t_i, int32_t nt, int64_t* nnz,
                       int32_t* indptr, int32_t* indices);
/* Vertex incidence of the matrix-free operator (no reference counterpart:
 * the reference assembles A in CSR): for each vertex v, entries
 * ptr[v] .. ptr[v+1]-1 hold 4 * t + l for every slot l of constraint t that
 * names v, in ascending t; a slot repeating a vertex of an earlier slot of
 * its constraint (a length constraint's a, b, a, b) is left out.  Vertex ids
 * must lie in [0, nv).  Call with ptr == NULL to get *n_entries, then again
 * with ptr (nv+1) and entries (*n_entries). */
int mgpbd_host_vertex_incidence(const int32_t* t_i, int32_t nt, int32_t nv, int64_t* n_entries,
                                int32_t* ptr, int32_t* entries);
/* tet_geometry_aggregation pass 1 (cons/tet_aggregation.py:40-127), with
 * the reference's tie order reproduced; agg_ids has nt entries. */
int mgpbd_host_aggregate(const int32_t* t_i, int32_t nt, int32_t max_agg_size,
                         int32_t* agg_ids, int32_t* n_agg);
/* build_tet_hierarchy (cons/tet_aggregation.py:145-211): level sizes
 * (sizes[0] = nt) and the level-0 aggregate ids; returns *n_levels (1 or 2). */
int mgpbd_host_tet_hierarchy(const int32_t* t_i, int32_t nt, int32_t max_coarse,
                             int32_t max_levels, int32_t* n_levels,
                             int32_t* sizes, int32_t* agg_ids);
/* Galerkin coarse pattern of P^T A P with scipy's exact-zero dropping and
 * the contribution map of cons/mgpcg_gpu.py:46-99 for piecewise-constant P.
 * Call with c_indptr == NULL to get *c_nnz and *n_contrib, then again with
 * c_indptr (n_agg+1), c_indices (*c_nnz), contrib_idx (*n_contrib) and
 * contrib_off (*c_nnz+1). */
int mgpbd_host_galerkin(int32_t n, const int32_t* indptr, const int32_t* indices,
                        const float* data, const int32_t* agg_ids, int32_t n_agg,
                        int64_t* c_nnz, int64_t* n_contrib, int32_t* c_indptr,
                        int32_t* c_indices, int32_t* contrib_idx,
                        int32_t* contrib_off);

/* The same Galerkin build on the GPU (one warp per coarse row, a float64
 * hash accumulation in the host build's summation order): bit-identical
 * outputs.  data == NULL gives the structural pattern (no value-based
 * dropping), the build used below the tet hierarchy.  Host arrays in and
 * out (copied to and from the device inside; the call blocks the host);
 * diag_pos (n_agg, -1 where a coarse row has no diagonal) may be NULL.
 * Replaces the host setup of cons/mgpcg_gpu.py:30-99; the solver's own
 * hierarchy build (mgpbd_init) uses this builder on the device arrays. */
int mgpbd_device_galerkin(int32_t n, const int32_t* indptr, const int32_t* indices,
                          const float* data, const int32_t* agg_ids, int32_t n_agg,
                          int64_t* c_nnz, int64_t* n_contrib, int32_t* c_indptr,
                          int32_t* c_indices, int32_t* contrib_idx, int32_t* contrib_off,
                          int32_t* diag_pos);

#ifdef __cplusplus
}
#endif

#endif /* MGPBD_H_ */
