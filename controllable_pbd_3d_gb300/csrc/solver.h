// The MGPBD solver object behind the C ABI (one body, one stream).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <memory>
#include <vector>

#include "bodies.cuh"
#include "common.h"
#include "jform.cuh"
#include "kernels.cuh"
#include "mpnn.cuh"
#include "rap.cuh"
#include "structure.h"

namespace mgpbd {

struct Level {
  int32_t n = 0;
  int64_t nnz = 0;
  DevBuf<int32_t> indptr, indices, diag_pos;
  DevBuf<float> data, diag_inv;
  // transfer to level+1 (absent on the coarsest level)
  DevBuf<int32_t> agg, mem_ptr, mem_rows;
  // Galerkin refill of this level from level-1 values (absent on level 0)
  DevBuf<int32_t> contrib_off, contrib_idx;
  // work vectors of the V-cycle
  DevBuf<float> b, xa, xb, r;
  // smoother weight used by the Jacobi sweeps of this level (device scalar)
  DevBuf<float> omega;
  // host copies of the structure (kept for the level below)
  Csr host;
  // tile shape of the vectorised row kernel on this level (-1: from the
  // mean row length; set by the autotuner or the caller)
  int shape = -1;
  CsrView view() const {
    CsrView v;
    v.n = n;
    v.nnz = nnz;
    v.indptr = indptr.p;
    v.indices = indices.p;
    v.data = data.p;
    v.diag_inv = diag_inv.p;
    v.padded = true;
    v.shape = shape;
    return v;
  }
};

class Solver {
 public:
  explicit Solver(const mgpbd_params& p);
  ~Solver();

  void set_stream(cudaStream_t s) { stream_ = s; }
  void set_mesh(const float* x_ref, const float* invm, const int32_t* t_i, int32_t nv, int32_t nt,
                float* x, float* v);
  void set_hierarchy(const int32_t* agg_ids, int32_t n_levels, const int32_t* level_sizes);
  // GPUMultigridSolver.setup (cons/mgpcg_gpu.py:30-173) for a caller's
  // level-0 matrix instead of a mesh: host CSR arrays, kept in the caller's
  // column order; init() then builds the coarse levels of the hierarchy
  // given by set_hierarchy (none: one level) and the V-cycle PCG solves it
  void set_matrix(int32_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                  const float* data);
  // update_fine_matrix_data + update_all_coarse_matrices (cons/mgpcg_gpu.py:
  // 175-212): new level-0 values (device, nnz), 1/diag and coarse refill
  void update_matrix(const float* data);
  // Independent bodies packed into the mesh (vertex ranges vert_off[b] ..
  // vert_off[b+1]; constraint ranges segs[3k] .. segs[3k+1] of body
  // segs[3k+2], covering [0, nt) in order): each body gets its own Newton
  // loop (residual, stopping test, line-search step) over one shared
  // block-diagonal CG solve per Newton iteration.  FAST Chebyshev only.
  void set_bodies(int32_t n_bodies, const int32_t* vert_off, int32_t n_segs, const int32_t* segs);
  int32_t n_bodies() const { return nb_; }
  // per body: Newton iterations, first and last residual, last line-search
  // step of the last solve
  void body_stats(int32_t n, int32_t* newton, double* r0, double* r, double* omega) const;
  // wait limit of the persistent CG kernels' grid barriers (seconds)
  void set_barrier_limit(double seconds) {
    require(seconds >= 0.0 && seconds <= 60.0, MGPBD_EINVAL, "barrier limit must be in [0, 60] s");
    barrier_limit_s_ = seconds;
  }
  // per-constraint MGPBD_CONS_* types (host array of nt; nullptr: all ARAP)
  void set_constraint_types(const int32_t* types);
  void init();
  void step(int32_t frame);
  void make_prediction();
  void solve(int32_t frame);
  void update_vel();

  // per-stage entry points
  void compute_constraints();
  void fill_matrices();
  void refill_coarse();
  double compute_rhs();
  int32_t pcg(const float* b, float* x);
  void vcycle_into(const float* r, float* z);
  void scatter(const float* dlam);
  double line_search();
  void apply_dpos(double omega);
  // matrix_free: 0 CSR values, 1 gradients (prepared first), 2 gradients
  // as prepared by the last call
  void apply_matrix(int matrix_free, const float* x, float* y);
  // adaptive zones (cons/adaptive_zone.py, cons/mgpbd_adaptive.py)
  void zone_proximity(int32_t* active, float cx, float cy, float cz, float radius);
  void zone_strain(int32_t* active, const float* x_old, float threshold, float dt);
  void zone_expand(int32_t* active, int32_t n_rings);
  void mask_alpha(const int32_t* active, float* saved);
  void restore_alpha(const float* saved);
  void level_sweep(int32_t level, int32_t op, const float* x, const float* b, float* y,
                   float omega);

  // row-kernel tile shapes per level: tune all levels (codes G*100+U and
  // the best time per Jacobi sweep), or read / set one level's
  void autotune_rows(int32_t reps, int32_t* codes, float* us);
  int32_t level_row_shape(int32_t l) const;
  void set_level_row_shape(int32_t l, int32_t code);

  // learned coarse correction (MGPBD_PRECOND_LEARNED)
  void set_coarse_net(CoarseNet* net) { net_ = net; }
  void record_coarse(float* rc, float* ec, int32_t capacity, int32_t every);
  int32_t record_count() const { return rec_count_; }

  const mgpbd_stats& stats() const { return stats_; }
  // rows of (iteration, residual, cg_iters, omega, host seconds) of the last
  // solve, one per call the reference makes to benchmark.record_iteration
  const std::vector<std::array<double, 5>>& newton_log() const { return log_; }
  uint32_t status() const { return status_; }
  void* field(int32_t id, int64_t* count);
  const Level& level(int32_t l) const;
  int32_t n_levels() const { return static_cast<int32_t>(levels_.size()); }
  cudaStream_t stream() const { return stream_; }

 private:
  void require_init() const;
  // packed bodies: per-body Newton loop, verified block-diagonal CG solve,
  // per-body sums over the constraint chunks
  void init_bodies(const std::vector<int32_t>& t_host);
  void solve_bodies();
  int32_t pcg_bodies(const float* b, float* x, const std::vector<double>& bnorm);
  void chunk_body_sums(int count, std::vector<double>& out);
  // the same loop as one captured CUDA graph per substep (use_graph)
  void solve_bodies_graph();
  void capture_body_graph();
  void drop_body_graph();
  BodyArrays body_arrays();
  BodyLimits body_limits() const;
  BodyCg body_cg();
  JcgVecs dual_vecs(const float* b, float* x);
  int32_t run_dual_bodies(const float* b, float* x, int32_t maxit, bool warm);
  int32_t run_dual(const float* b, float* x, double tol_abs, double tol_rel, int32_t maxit,
                   bool warm, float4* ulo);
  // the per-mesh stages need set_mesh (not a caller's matrix)
  void require_mesh() const;
  void init_matrix();
  void build_hierarchy(const std::vector<int32_t>& t_i_host);
  void push_coarse(DeviceGalerkin& g, int32_t n_agg);
  void alloc_work();
  // V-cycle on `l` with rhs b_l (device) and zero initial guess; the result
  // is left in levels_[l].xa.
  void vcycle(int32_t l, const float* b, const CgState* guard);
  void smooth_level(int32_t l, const float* b, float*& cur, float*& nxt, int sweeps,
                    bool from_zero, const CgState* guard);
  void update_smoother_weights();
  void factor_coarsest();
  void cg_body(const float* b, float* x);
  // z = V-cycle(r) for the CG residual r (level-0 result left in xa)
  void precondition(const CgState* guard);
  int32_t pcg_graph(const float* b, float* x);
  // PCG with the learned coarse correction, judged and backed up by the
  // plain V-cycle
  bool learned() const { return p_.precond == MGPBD_PRECOND_LEARNED; }
  int32_t pcg_learned(const float* b, float* x);
  // coarse correction of the level-0 V-cycle into levels_[1].xa
  void coarse_correction(const CgState* guard);
  NetGraph net_graph() const;
  // 1/2 e^T A_1 e - e^T r on level 1 (host sync)
  double coarse_energy(const float* e, const float* r);
  // FAST mode with the Chebyshev preconditioner (matrix-free A)
  bool cheb() const { return p_.precond == MGPBD_PRECOND_CHEB; }
  JView jview();
  JVecs jvecs(const float* b, float* x);
  void jform_setup(uint32_t* dev_status = nullptr);
  int32_t pcg_cheb(const float* b, float* x);
  void sync_read(void* host, const void* dev, size_t bytes);
  double finalize_read(const double* partials, int blocks);

  mgpbd_params p_;
  cudaStream_t stream_ = nullptr;
  const float* x_ref_ = nullptr;
  const float* invm_ = nullptr;
  const int32_t* t_i_ = nullptr;
  float* x_ = nullptr;
  float* v_ = nullptr;
  int32_t nv_ = 0, nt_ = 0;
  bool inited_ = false;
  bool matrix_mode_ = false;     // set_matrix: a caller's level-0 matrix, no mesh
  double barrier_limit_s_ = 4.0; // grid-barrier wait limit of the persistent kernels
  const float* dual_x_ = nullptr;  // x of the last persistent dual solve (its low part in jxc_)
  // warm_substep: the first solution of the last substep, and whether the
  // next dual solve starts from what x holds
  DevBuf<float> dlam_prev_;
  bool have_prev_ = false;
  bool warm_next_ = false;
  // packed bodies (set_bodies)
  int32_t nb_ = 0;
  std::vector<int32_t> body_vert_off_, body_segs_, chunk_body_;
  DevBuf<int32_t> chunks_, cons_body_, vert_body_, body_active_;
  DevBuf<float> body_omega_;
  DevBuf<double> chunk_partials_;
  DevBuf<float4> ulo_;  // warm restarts of the dual CG: low parts of u (float64 residual)
  std::vector<int32_t> body_newton_;
  std::vector<double> body_r0_, body_r_, body_omega_h_;
  // device side of the loop for the captured substep (bodies.cuh)
  DevBuf<int32_t> body_chunk_ptr_, body_chunk_idx_, body_newton_d_;
  DevBuf<double> body_r0_d_, body_r_d_, body_bnorm_d_, body_sq_d_, body_cur_d_, body_omh_d_;
  DevBuf<BodyLoop> body_loop_;
  DevBuf<BodyLogEntry> body_log_;
  BodyLoop* h_body_loop_ = nullptr;  // pinned
  // per-body CG (body_cg): chunks of at most 256 constraints inside one body
  DevBuf<int32_t> bcg_ch_, bcg_chb_, bcg_bptr_, bcg_bidx_, bcg_done_, bcg_iters_;
  DevBuf<double> bcg_cp_, bcg_sc_;
  DevBuf<float> bcg_fa_, bcg_fb_;
  DevBuf<uint32_t> bcg_ndone_;
  DevBuf<int32_t> body_have_prev_;  // warm_substep: dlam_prev_ holds a solution
  cudaGraphExec_t body_exec_ = nullptr;
  double body_exec_limit_ = -1.0;  // barrier limit baked into the captured launches
  long long body_graph_init_launches_ = 0, body_graph_body_launches_ = 0;
  Csr mat_csr_;                  // its structure and values (host)
  std::vector<float> mat_vals_;

  DevBuf<float> x_old_, x_pred_, dpos_;
  DevBuf<float> dm_inv_, rest_vol_, alpha_, lambda_, C_, gradC_, rhs_, dlam_;
  DevBuf<int32_t> inc_ptr_, inc_ent_;
  int64_t inc_n_ = 0;                  // incidence entries
  int32_t n4_ = 0;                     // first trailing length constraint (nt_: none)
  DevBuf<float4> gE_;                  // their gradients n
  DevBuf<int32_t> qE_;                 // their vertex pairs
  DevBuf<int32_t> ctype_;              // constraint types (absent: all ARAP)
  std::vector<int32_t> ctype_host_;
  std::vector<Level> levels_;

  DevBuf<float> cg_r_, cg_z_, cg_p_, cg_ap_;
  DevBuf<double> partials_, scalars_, omegas_;
  DevBuf<CgState> cg_state_;
  DevBuf<double> chol_;
  DevBuf<int32_t> chol_info_;
  DevBuf<float> pw_a_, pw_b_;  // power-iteration vectors
  double* h_buf_ = nullptr;    // pinned host scratch
  CgState* h_state_ = nullptr;
  ChebCoef* h_cf_ = nullptr;   // pinned staging of the Chebyshev coefficients
  cudaEvent_t ev_[2] = {nullptr, nullptr};  // around each persistent CG launch
  static double event_ms(cudaEvent_t a, cudaEvent_t b);

  // captured CG loop (FAST mode)
  cudaGraphExec_t cg_exec_ = nullptr;
  const float* cg_graph_b_ = nullptr;
  float* cg_graph_x_ = nullptr;
  long long graph_init_launches_ = 0;
  long long graph_body_launches_ = 0;

  // matrix-free (J-form) data of the Chebyshev path
  DevBuf<float4> gV_, u_;
  DevBuf<float> jdinv_, jz_, jd_, jp_, jap_, pw_v_, pw_w_;
  DevBuf<double> jxd_, jr_;
  DevBuf<JState> jst_;
  DevBuf<float> jxc_, jrf_;  // persistent CG: Kahan term of x, float32 residual
  DevBuf<GridSync> jgs_;
  DevBuf<int32_t> adj_ptr_, adj_, zone_scratch_;  // face adjacency (built on first use)
  DevBuf<float4> gT_;      // persistent CG: gradients as three planes
  JcgPlan jplan_;          // persistent CG work split
  std::vector<int32_t> user_sizes_;               // mgpbd_set_hierarchy
  std::vector<std::vector<int32_t>> user_aggs_;
  JcgPlan pplan_;          // the same for the primal warm start
  DevBuf<float4> pv_[10];  // primal CG vertex vectors
  DevBuf<float> ps_;       // primal CG tet scratch
  bool primal() const { return cheb() && p_.persistent && p_.primal; }
  DevBuf<int32_t> jpart_;  // jplan_.vb then jplan_.tb
  cudaGraphExec_t jcg_exec_ = nullptr;
  const float* jcg_b_ = nullptr;
  float* jcg_x_ = nullptr;
  long long jgraph_init_launches_ = 0;
  long long jgraph_body_launches_ = 0;

  CoarseNet* net_ = nullptr;
  bool net_active_ = false;   // the current solve uses the network
  bool judge_pending_ = false;
  DevBuf<float> net_e_, net_t_, net_w_;
  float* rec_rc_ = nullptr;
  float* rec_ec_ = nullptr;
  int32_t rec_cap_ = 0, rec_every_ = 1, rec_count_ = 0;
  int64_t rec_calls_ = 0;

  mgpbd_stats stats_{};
  uint32_t status_ = 0;
  std::vector<std::array<double, 5>> log_;
};

}  // namespace mgpbd
