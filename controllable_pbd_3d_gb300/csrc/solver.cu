// MGPBD solver: the Newton loop of MGPBDSolverGPU (cons/mgpbd_gpu.py:397-446)
// around the multigrid-preconditioned CG of GPUMultigridSolver
// (cons/mgpcg_gpu.py:214-329), on one CUDA stream.
#include "solver.h"
#include "zone.cuh"

#include <algorithm>
#include <limits>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>

namespace mgpbd {

namespace {

template <class T>
void upload(DevBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  d.alloc(static_cast<int64_t>(h.size()));
  if (!h.empty())
    MGPBD_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s));
}

// CSR value/index arrays get kCsrPad zeroed elements after the last entry so
// the vectorised row kernel's last 16-byte window stays inside the buffer.
template <class T>
void alloc_padded(DevBuf<T>& d, int64_t n, cudaStream_t s) {
  d.alloc(n + kCsrPad);
  MGPBD_CUDA(cudaMemsetAsync(d.p, 0, sizeof(T) * (n + kCsrPad), s));
}

template <class T>
void upload_padded(DevBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  alloc_padded(d, static_cast<int64_t>(h.size()), s);
  if (!h.empty())
    MGPBD_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s));
}

// Power-iteration estimate of lambda_max(D^-1 A); the weight written to
// *omega is min(omega_cap, 4 / (3 * 1.1 * lambda)).
__global__ void k_pw_init(float* v, int32_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = static_cast<uint32_t>(i) * 2654435761u;
    h ^= h >> 15;
    v[i] = 0.5f + (h & 0xffff) * (1.0f / 65536.0f);
  }
}

__global__ void k_pw_step(int32_t n, const int32_t* __restrict__ indptr,
                          const int32_t* __restrict__ indices, const float* __restrict__ data,
                          const float* __restrict__ dinv, const float* __restrict__ x,
                          float* __restrict__ y, double* __restrict__ partials) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) s += data[k] * x[indices[k]];
    float v = dinv[i] * s;
    y[i] = v;
    acc += (double)v * v;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
  }
}

__global__ void k_pw_scale(float* __restrict__ v, int32_t n, const double* __restrict__ nrm2) {
  double s = nrm2[0];
  float inv = s > 0.0 ? (float)(1.0 / sqrt(s)) : 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= inv;
}

__global__ void k_pw_weight(const double* __restrict__ nrm2, float omega_cap, float* omega) {
  double lam = sqrt(nrm2[0]);
  float w = omega_cap;
  if (lam > 0.0 && isfinite(lam)) {
    float safe = (float)(4.0 / (3.0 * 1.1 * lam));
    w = safe < omega_cap ? safe : omega_cap;
  }
  *omega = w;
}

__global__ void k_set_cond(cudaGraphConditionalHandle h, CgState* st) {
  st->body_runs += 1;
  cudaGraphSetConditional(h, st->done ? 0u : 1u);
}

__global__ void k_fill_f32(float* p, float v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

}  // namespace

Solver::Solver(const mgpbd_params& p) : p_(p) {
  require(p.dt > 0.0f, MGPBD_EINVAL, "dt must be positive");
  require(p.n_smooth >= 0 && p.maxiter >= 0 && p.maxiter_cg >= 0, MGPBD_EINVAL,
          "iteration counts must be non-negative");
  require(p.mode == MGPBD_MODE_PARITY || p.mode == MGPBD_MODE_FAST, MGPBD_EINVAL, "unknown mode");
  require(p.persistent >= 0 && p.persistent <= 2, MGPBD_EINVAL, "persistent must be 0, 1 or 2");
  require(p.precond == MGPBD_PRECOND_VCYCLE || p.precond == MGPBD_PRECOND_CHEB ||
              p.precond == MGPBD_PRECOND_LEARNED,
          MGPBD_EINVAL, "unknown preconditioner");
  if (p.precond == MGPBD_PRECOND_LEARNED) {
    require(!p.cg_alias, MGPBD_EINVAL, "cg_alias does not combine with the learned coarse correction");
    require(p.learned_stall >= 0, MGPBD_EINVAL, "learned_stall must be non-negative");
  }
  if (p.precond == MGPBD_PRECOND_CHEB) {
    require(p.mode == MGPBD_MODE_FAST, MGPBD_EINVAL, "the Chebyshev preconditioner needs FAST mode");
    require(p.cheb_degree >= 1 && p.cheb_degree < kMaxCheb, MGPBD_EINVAL,
            "cheb_degree must be in [1, 31]");
    require(p.cheb_lo > 0.0f && p.cheb_lo < 1.0f, MGPBD_EINVAL, "cheb_lo must be in (0, 1)");
    require(!p.cg_alias, MGPBD_EINVAL, "cg_alias applies to the V-cycle preconditioner only");
  }
  // no CUDA call here: a handle can be created (and its host-side
  // validation exercised) on a machine without a GPU
}

Solver::~Solver() {
  if (cg_exec_) cudaGraphExecDestroy(cg_exec_);
  if (jcg_exec_) cudaGraphExecDestroy(jcg_exec_);
  if (body_exec_) cudaGraphExecDestroy(body_exec_);
  if (h_body_loop_) cudaFreeHost(h_body_loop_);
  if (h_buf_) cudaFreeHost(h_buf_);
  if (h_state_) cudaFreeHost(h_state_);
  if (h_cf_) cudaFreeHost(h_cf_);
  for (cudaEvent_t e : ev_)
    if (e) cudaEventDestroy(e);
}

// elapsed time between two events recorded on the solver stream, once the
// second has completed (the callers have synchronised)
double Solver::event_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  MGPBD_CUDA(cudaEventElapsedTime(&ms, a, b));
  return ms;
}

void Solver::require_init() const {
  require(inited_, MGPBD_ESTATE, "mgpbd_init has not been called");
}

void Solver::require_mesh() const {
  require_init();
  require(!matrix_mode_, MGPBD_ESTATE,
          "this handle solves a caller's matrix (mgpbd_set_matrix): it has no mesh");
}

void Solver::set_matrix(int32_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                        const float* data) {
  require(indptr && indices && data, MGPBD_EINVAL, "null matrix array");
  require(n > 0 && nnz > 0, MGPBD_EINVAL, "empty matrix");
  require(nnz < INT32_MAX, MGPBD_ERANGE, "too many nonzeros for int32 row pointers");
  require(indptr[0] == 0 && indptr[n] == nnz, MGPBD_EINVAL, "indptr must run from 0 to nnz");
  for (int32_t i = 0; i < n; ++i) {
    require(indptr[i + 1] >= indptr[i], MGPBD_EINVAL, "indptr must not decrease");
    bool diag = false;
    for (int64_t k = indptr[i]; k < indptr[i + 1]; ++k) {
      require(indices[k] >= 0 && indices[k] < n, MGPBD_EINVAL, "column index outside [0, n)");
      diag |= indices[k] == i;
    }
    require(diag, MGPBD_EINVAL, "every row needs its diagonal entry (Jacobi smoother)");
  }
  x_ref_ = invm_ = nullptr;
  t_i_ = nullptr;
  x_ = v_ = nullptr;
  nv_ = 0;
  nt_ = n;
  mat_csr_.n_rows = mat_csr_.n_cols = n;
  mat_csr_.indptr.assign(indptr, indptr + n + 1);
  mat_csr_.indices.assign(indices, indices + nnz);
  mat_vals_.assign(data, data + nnz);
  matrix_mode_ = true;
  inited_ = false;
  user_sizes_.clear();
  user_aggs_.clear();
  ctype_host_.clear();
  if (cg_exec_) {
    cudaGraphExecDestroy(cg_exec_);
    cg_exec_ = nullptr;
  }
}

void Solver::update_matrix(const float* data) {
  require_init();
  require(matrix_mode_, MGPBD_ESTATE, "mgpbd_update_matrix needs mgpbd_set_matrix");
  require(data != nullptr, MGPBD_EINVAL, "null values");
  Level& L0 = levels_[0];
  MGPBD_CUDA(cudaMemcpyAsync(L0.data.p, data, sizeof(float) * L0.nnz, cudaMemcpyDeviceToDevice,
                             stream_));
  launch_diag_inv_scan(L0.indptr.p, L0.indices.p, L0.data.p, L0.n, L0.diag_inv.p, stream_);
  refill_coarse();
}

void Solver::init_matrix() {
  require(!cheb() && !learned(), MGPBD_ENOTSUP,
          "a caller's matrix is solved by the V-cycle PCG (precond vcycle)");
  cudaStream_t s = stream_;
  if (!h_buf_) MGPBD_CUDA(cudaMallocHost(&h_buf_, sizeof(double) * 64));
  if (!h_state_) MGPBD_CUDA(cudaMallocHost(&h_state_, sizeof(CgState)));
  if (!h_cf_) MGPBD_CUDA(cudaMallocHost(&h_cf_, sizeof(ChebCoef)));
  for (cudaEvent_t& e : ev_)
    if (!e) MGPBD_CUDA(cudaEventCreate(&e));
  partials_.alloc(static_cast<int64_t>(kMaxReduceBlocks) * 16);
  scalars_.alloc(64);
  omegas_.alloc(16);
  cg_state_.alloc(1);
  levels_.clear();
  levels_.emplace_back();
  Level& L0 = levels_[0];
  L0.host = mat_csr_;
  L0.n = nt_;
  L0.nnz = L0.host.nnz();
  upload(L0.indptr, L0.host.indptr, s);
  upload_padded(L0.indices, L0.host.indices, s);
  upload_padded(L0.data, mat_vals_, s);
  L0.diag_inv.alloc(nt_);
  launch_diag_inv_scan(L0.indptr.p, L0.indices.p, L0.data.p, L0.n, L0.diag_inv.p, s);
  build_hierarchy({});
  alloc_work();
  inited_ = true;
  refill_coarse();
  MGPBD_CUDA(cudaStreamSynchronize(s));
  stats_ = mgpbd_stats{};
  stats_.n_levels = n_levels();
  for (int32_t l = 0; l < n_levels() && l < 8; ++l) {
    stats_.rows[l] = levels_[l].n;
    stats_.nnz[l] = levels_[l].nnz;
  }
}

// Caller-provided aggregation hierarchy (used by the next init instead of
// the built-in tet aggregation): level_sizes[0] = nt, and for each level l
// the level_sizes[l] entries of agg_ids from offset sum(level_sizes[0..l))
// map level-l rows onto [0, level_sizes[l+1]), every coarse row used.
void Solver::set_constraint_types(const int32_t* types) {
  require(t_i_ != nullptr, MGPBD_ESTATE, "mgpbd_set_mesh has not been called");
  if (!types) {
    ctype_host_.clear();
  } else {
    ctype_host_.assign(types, types + nt_);
  }
  inited_ = false;
}

void Solver::set_hierarchy(const int32_t* agg_ids, int32_t n_levels, const int32_t* level_sizes) {
  require((x_ && t_i_) || matrix_mode_, MGPBD_ESTATE,
          "mgpbd_set_mesh or mgpbd_set_matrix must come before mgpbd_set_hierarchy");
  require(n_levels >= 2 && n_levels <= 8, MGPBD_EINVAL, "n_levels must be in [2, 8]");
  require(level_sizes != nullptr && agg_ids != nullptr, MGPBD_EINVAL, "null hierarchy array");
  require(level_sizes[0] == nt_, MGPBD_EINVAL, "level_sizes[0] must equal nt");
  std::vector<int32_t> sizes(level_sizes, level_sizes + n_levels);
  std::vector<std::vector<int32_t>> aggs;
  int64_t off = 0;
  for (int32_t l = 0; l + 1 < n_levels; ++l) {
    require(sizes[l + 1] >= 1 && sizes[l + 1] <= sizes[l], MGPBD_EINVAL,
            "each level must be smaller than the one above");
    std::vector<int32_t> a(agg_ids + off, agg_ids + off + sizes[l]);
    std::vector<uint8_t> used(sizes[l + 1], 0);
    for (int32_t v : a) {
      require(v >= 0 && v < sizes[l + 1], MGPBD_EINVAL, "aggregate id out of range");
      used[v] = 1;
    }
    for (uint8_t u : used) require(u != 0, MGPBD_EINVAL, "empty aggregate");
    aggs.push_back(std::move(a));
    off += sizes[l];
  }
  user_sizes_ = std::move(sizes);
  user_aggs_ = std::move(aggs);
  inited_ = false;
}

void Solver::set_mesh(const float* x_ref, const float* invm, const int32_t* t_i, int32_t nv,
                      int32_t nt, float* x, float* v) {
  require(x_ref && invm && t_i && x && v, MGPBD_EINVAL, "null mesh pointer");
  require(nv > 0 && nt > 0, MGPBD_EINVAL, "empty mesh");
  require(static_cast<int64_t>(nt) * 4 < INT32_MAX, MGPBD_ERANGE, "too many tets for int32 indices");
  x_ref_ = x_ref;
  invm_ = invm;
  t_i_ = t_i;
  nv_ = nv;
  nt_ = nt;
  x_ = x;
  v_ = v;
  matrix_mode_ = false;
  nb_ = 0;
  inited_ = false;
  user_sizes_.clear();
  user_aggs_.clear();
  ctype_host_.clear();
  if (cg_exec_) {
    cudaGraphExecDestroy(cg_exec_);
    cg_exec_ = nullptr;
  }
  if (jcg_exec_) {
    cudaGraphExecDestroy(jcg_exec_);
    jcg_exec_ = nullptr;
  }
  drop_body_graph();
  have_prev_ = false;
}

void Solver::sync_read(void* host, const void* dev, size_t bytes) {
  MGPBD_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, stream_));
  MGPBD_CUDA(cudaStreamSynchronize(stream_));
}

double Solver::finalize_read(const double* partials, int blocks) {
  launch_finalize(partials, blocks, 1, scalars_.p, stream_);
  sync_read(h_buf_, scalars_.p, sizeof(double));
  return h_buf_[0];
}

// ---------------------------------------------------------------------------
// MGPBDSolverGPU.init (cons/mgpbd_gpu.py:92-114)
void Solver::init() {
  have_prev_ = false;
  if (matrix_mode_) {
    init_matrix();
    return;
  }
  require(x_ && t_i_, MGPBD_ESTATE, "mgpbd_set_mesh has not been called");
  cudaStream_t s = stream_;
  if (!h_buf_) MGPBD_CUDA(cudaMallocHost(&h_buf_, sizeof(double) * 64));
  if (!h_state_) MGPBD_CUDA(cudaMallocHost(&h_state_, sizeof(CgState)));
  if (!h_cf_) MGPBD_CUDA(cudaMallocHost(&h_cf_, sizeof(ChebCoef)));
  for (cudaEvent_t& e : ev_)
    if (!e) MGPBD_CUDA(cudaEventCreate(&e));
  x_old_.alloc(3LL * nv_);
  x_pred_.alloc(3LL * nv_);
  dpos_.alloc(3LL * nv_);
  dm_inv_.alloc(9LL * nt_);
  rest_vol_.alloc(nt_);
  alpha_.alloc(nt_);
  lambda_.alloc(nt_);
  C_.alloc(nt_);
  gradC_.alloc(12LL * nt_);
  rhs_.alloc(nt_);
  dlam_.alloc(nt_);
  MGPBD_CUDA(cudaMemsetAsync(lambda_.p, 0, sizeof(float) * nt_, s));
  MGPBD_CUDA(cudaMemsetAsync(dpos_.p, 0, sizeof(float) * 3 * nv_, s));
  MGPBD_CUDA(cudaMemsetAsync(x_old_.p, 0, sizeof(float) * 3 * nv_, s));
  MGPBD_CUDA(cudaMemsetAsync(x_pred_.p, 0, sizeof(float) * 3 * nv_, s));
  partials_.alloc(static_cast<int64_t>(kMaxReduceBlocks) * 16);
  scalars_.alloc(64);
  omegas_.alloc(16);
  cg_state_.alloc(1);

  // validate every vertex id before any kernel gathers through t_i
  std::vector<int32_t> t_host(4LL * nt_);
  MGPBD_CUDA(cudaMemcpyAsync(t_host.data(), t_i_, sizeof(int32_t) * t_host.size(),
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
  for (int32_t v : t_host)
    require(v >= 0 && v < nv_, MGPBD_EINVAL, "t_i holds a vertex id outside [0, nv)");
  require((reinterpret_cast<uintptr_t>(t_i_) & 15) == 0 && (reinterpret_cast<uintptr_t>(x_) & 3) == 0,
          MGPBD_EINVAL, "t_i must be 16-byte aligned (read as int4)");

  // constraint types (mgpbd_set_constraint_types): a length constraint lists
  // its edge twice (a, b, a, b) and needs compliance-based alpha~
  ctype_.release();
  if (!ctype_host_.empty()) {
    require(static_cast<int64_t>(ctype_host_.size()) == nt_, MGPBD_EINVAL,
            "constraint types: one per constraint (nt)");
    bool generic = false;
    for (int32_t c = 0; c < nt_; ++c) {
      const int32_t ty = ctype_host_[c];
      require(ty == MGPBD_CONS_ARAP || ty == MGPBD_CONS_LENGTH || ty == MGPBD_CONS_VOLUME,
              MGPBD_EINVAL, "unknown constraint type");
      generic |= ty != MGPBD_CONS_ARAP;
      if (ty == MGPBD_CONS_LENGTH) {
        const int32_t* q = t_host.data() + 4LL * c;
        require(q[2] == q[0] && q[3] == q[1] && q[0] != q[1], MGPBD_EINVAL,
                "a length constraint must list its two vertices twice: (a, b, a, b)");
      }
    }
    require(!generic || p_.compliance > 0.0f, MGPBD_EINVAL,
            "length and volume constraints take alpha~ = compliance / dt^2: set compliance > 0");
    ctype_.alloc(nt_);
    MGPBD_CUDA(cudaMemcpyAsync(ctype_.p, ctype_host_.data(), sizeof(int32_t) * nt_,
                               cudaMemcpyHostToDevice, s));
  }
  launch_rest_shape(x_ref_, t_i_, ctype_.p, nt_,
                    p_.compliance > 0.0f ? -p_.compliance : p_.mu, p_.dt, dm_inv_.p, rest_vol_.p,
                    alpha_.p, s);

  // level-0 pattern (cons/mgpbd_gpu.py:153-194)
  levels_.clear();
  levels_.emplace_back();
  Level& L0 = levels_[0];
  L0.host = build_pattern(t_host.data(), nt_);
  L0.n = nt_;
  L0.nnz = L0.host.nnz();
  upload(L0.indptr, L0.host.indptr, s);
  upload_padded(L0.indices, L0.host.indices, s);
  alloc_padded(L0.data, L0.nnz, s);
  L0.diag_inv.alloc(nt_);

  std::vector<int32_t> ip, ie;
  vertex_incidence(t_host.data(), nt_, nv_, ip, ie);
  upload(inc_ptr_, ip, s);
  upload(inc_ent_, ie, s);
  inc_n_ = static_cast<int64_t>(ie.size());
  // trailing length constraints in compact form (gradient n, two vertices)
  // for the unstaged tet phases of the persistent kernels
  n4_ = nt_;
  gE_.release();
  qE_.release();
  if (cheb() && p_.persistent && !ctype_host_.empty()) {
    int32_t n4 = nt_;
    while (n4 > 0 && ctype_host_[n4 - 1] == MGPBD_CONS_LENGTH) --n4;
    if (n4 < nt_) {
      std::vector<int32_t> qe(2LL * (nt_ - n4));
      for (int32_t c = n4; c < nt_; ++c) {
        qe[2LL * (c - n4)] = t_host[4LL * c];
        qe[2LL * (c - n4) + 1] = t_host[4LL * c + 1];
      }
      upload(qE_, qe, s);
      gE_.alloc(nt_ - n4);
      n4_ = n4;
    }
  }
  if (cheb() && p_.persistent) {
    jplan_ = jcg_plan(ip, nv_, nt_, p_.persistent != 2);
    if (primal()) {
      pplan_ = jplan_;
      if (!pplan_.staged || !pcg_plan_fits(pplan_)) {
        pplan_.staged = false;
        pplan_.grid = pcg_unstaged_grid();
      }
    }
    if (jplan_.staged) {
      std::vector<int32_t> part(jplan_.vb);
      part.insert(part.end(), jplan_.tb.begin(), jplan_.tb.end());
      upload(jpart_, part, s);
    }
  }

  // first A at the current positions (cons/mgpbd_gpu.py:98-100)
  launch_constraints(x_, t_i_, ctype_.p, dm_inv_.p, rest_vol_.p, nt_, C_.p, gradC_.p, s);
  launch_fill_A(L0.indptr.p, L0.indices.p, t_i_, invm_, gradC_.p, alpha_.p, nt_, L0.data.p,
                L0.diag_inv.p, s);
  build_hierarchy(t_host);
  alloc_work();
  MGPBD_CUDA(cudaStreamSynchronize(s));
  inited_ = true;
  stats_ = mgpbd_stats{};
  stats_.n_levels = n_levels();
  if (cheb() && p_.persistent) {
    stats_.cg_path = jplan_.staged ? MGPBD_CGPATH_STAGED : MGPBD_CGPATH_PERSISTENT;
    if (primal())
      stats_.cg_path = pplan_.staged ? MGPBD_CGPATH_PRIMAL_STAGED : MGPBD_CGPATH_PRIMAL;
    stats_.cg_grid = jplan_.grid;
  }
  for (int32_t l = 0; l < n_levels() && l < 8; ++l) {
    stats_.rows[l] = levels_[l].n;
    stats_.nnz[l] = levels_[l].nnz;
  }
  if (nb_ > 0) {
    inited_ = false;
    init_bodies(t_host);
    inited_ = true;
  }
}

// Transfer maps of level l (aggregate id per row, the members of each
// aggregate ascending) uploaded to the level.
static void upload_transfer(Level& F, const std::vector<int32_t>& agg, int32_t n_agg,
                            cudaStream_t s) {
  std::vector<int32_t> mp(n_agg + 1, 0), mr(F.n);
  for (int32_t i = 0; i < F.n; ++i) mp[agg[i] + 1]++;
  for (int32_t a = 0; a < n_agg; ++a) mp[a + 1] += mp[a];
  std::vector<int32_t> cur(mp.begin(), mp.end() - 1);
  for (int32_t i = 0; i < F.n; ++i) mr[cur[agg[i]]++] = i;
  upload(F.agg, agg, s);
  upload(F.mem_ptr, mp, s);
  upload(F.mem_rows, mr, s);
}

// The coarse level below levels_.back() from its device Galerkin build.
void Solver::push_coarse(DeviceGalerkin& g, int32_t n_agg) {
  cudaStream_t s = stream_;
  levels_.emplace_back();
  Level& C = levels_.back();
  C.n = n_agg;
  C.nnz = g.nnz;
  C.indptr = std::move(g.indptr);
  C.indices = std::move(g.indices);  // kCsrPad zeroed entries after the last
  C.diag_pos = std::move(g.diag_pos);
  C.contrib_off = std::move(g.contrib_off);
  C.contrib_idx = std::move(g.contrib_idx);
  alloc_padded(C.data, C.nnz, s);
  C.diag_inv.alloc(C.n);
  C.host.n_rows = C.host.n_cols = n_agg;
  C.host.indptr = std::move(g.host_indptr);
  C.host.indices = std::move(g.host_indices);
}

void Solver::build_hierarchy(const std::vector<int32_t>& t_host) {
  cudaStream_t s = stream_;
  int32_t max_coarse = p_.max_coarse > 0 ? p_.max_coarse : 400;
  // tet hierarchy (cons/tet_aggregation.py:145-211, max_levels = 4)
  std::vector<int32_t> sizes;
  std::vector<std::vector<int32_t>> aggs;
  if (!user_sizes_.empty()) {
    sizes = user_sizes_;
    aggs = user_aggs_;
  } else if (!matrix_mode_) {
    tet_hierarchy(t_host.data(), nt_, max_coarse, 4, sizes, aggs);
  }
  // Galerkin levels from the values on the device (level 0: the first A);
  // each new level's values are refilled at once for the level after it
  for (size_t l = 0; l < aggs.size(); ++l) {
    const int32_t n_agg = sizes[l + 1];
    Level& F = levels_[l];
    upload_transfer(F, aggs[l], n_agg, s);
    DeviceGalerkin g;
    galerkin_device(F.n, F.nnz, F.indptr.p, F.indices.p, F.data.p, F.agg.p, F.mem_ptr.p,
                    F.mem_rows.p, n_agg, g, s);
    push_coarse(g, n_agg);
    Level& C = levels_.back();
    launch_rap_refill(C.contrib_off.p, C.contrib_idx.p, levels_[l].data.p, C.nnz, C.data.p, s);
  }
  // optional extra levels by matrix-graph aggregation (not in the reference,
  // whose tet hierarchy stops at two levels)
  int32_t extra = 0;
  while (extra < p_.max_levels && levels_.back().n > max_coarse) {
    Level& F = levels_.back();
    std::vector<int32_t> agg;
    int32_t n_agg = graph_aggregate(F.host, 8, agg);
    if (n_agg >= F.n || n_agg <= 0) break;
    upload_transfer(F, agg, n_agg, s);
    DeviceGalerkin g;
    galerkin_device(F.n, F.nnz, F.indptr.p, F.indices.p, nullptr, F.agg.p, F.mem_ptr.p,
                    F.mem_rows.p, n_agg, g, s);
    push_coarse(g, n_agg);
    ++extra;
  }
  require(levels_.size() <= 8, MGPBD_ERANGE, "more than 8 multigrid levels");
}

void Solver::alloc_work() {
  cudaStream_t s = stream_;
  for (Level& L : levels_) {
    L.b.alloc(L.n);
    L.xa.alloc(L.n);
    L.xb.alloc(L.n);
    L.r.alloc(L.n);
    L.omega.alloc(1);
    k_fill_f32<<<1, 32, 0, s>>>(L.omega.p, p_.omega_jacobi, 1);
    MGPBD_CHECK_LAUNCH();
  }
  cg_r_.alloc(nt_);
  cg_z_.alloc(nt_);
  cg_p_.alloc(nt_);
  cg_ap_.alloc(nt_);
  if (p_.smoother == MGPBD_SMOOTH_JACOBI_SAFE) {
    int32_t nmax = 0;
    for (Level& L : levels_) nmax = std::max(nmax, L.n);
    pw_a_.alloc(static_cast<int64_t>(nmax) * levels_.size());
    pw_b_.alloc(nmax);
    int64_t off = 0;
    for (Level& L : levels_) {
      k_pw_init<<<std::max(1, ceil_div(L.n, 256)), 256, 0, s>>>(pw_a_.p + off, L.n);
      MGPBD_CHECK_LAUNCH();
      off += nmax;
    }
  }
  if (p_.coarse_solver == MGPBD_COARSE_DENSE_F64) {
    int32_t n = levels_.back().n;
    require(n <= 4096, MGPBD_ERANGE, "coarsest level too large for the dense solve");
    chol_.alloc(static_cast<int64_t>(n) * n);
    chol_info_.alloc(1);
  }
  // matrix-free operator data (used by the Chebyshev path and by
  // mgpbd_apply_matrix in every mode)
  if (matrix_mode_) return;  // a caller's matrix has no operator data
  gV_.alloc(4LL * nt_);
  u_.alloc(nv_);
  jdinv_.alloc(nt_);
  MGPBD_CUDA(cudaMemsetAsync(u_.p, 0, sizeof(float4) * nv_, s));
  if (cheb()) {
    jz_.alloc(nt_);
    jd_.alloc(nt_);
    jp_.alloc(nt_);
    jap_.alloc(nt_);
    pw_v_.alloc(nt_);
    pw_w_.alloc(nt_);
    jxd_.alloc(nt_);
    jr_.alloc(nt_);
    jst_.alloc(1);
    MGPBD_CUDA(cudaMemsetAsync(jst_.p, 0, sizeof(JState), s));
    jxc_.alloc(nt_);
    jrf_.alloc(nt_);
    jgs_.alloc(1);
    if (p_.persistent) {
      gT_.alloc(3LL * nt_);
      ulo_.alloc(nv_);
      MGPBD_CUDA(cudaMemsetAsync(ulo_.p, 0, sizeof(float4) * nv_, s));
    }
    if (primal()) {
      for (auto& b : pv_) {
        b.alloc(nv_);
        MGPBD_CUDA(cudaMemsetAsync(b.p, 0, sizeof(float4) * nv_, s));
      }
      ps_.alloc(nt_);
    }
    launch_seed(pw_v_.p, nt_, s);
  }
}

// y = A x on level 0: matrix-free from the current gradients, or the CSR
// values of the last fill
void Solver::apply_matrix(int matrix_free, const float* x, float* y) {
  require_mesh();
  if (matrix_free) {
    JView j = jview();
    if (matrix_free == 1)
      launch_jform_prepare(j, inc_ent_.p, gV_.p, jdinv_.p, gT_.p,
                           p_.cheb_scale == MGPBD_CHEB_UNSCALED, stream_);
    launch_jform_apply(j, x, y, stream_);
  } else {
    launch_spmv(levels_[0].view(), x, y, stream_);
  }
}

// ---- adaptive zones ------------------------------------------------------
void Solver::zone_proximity(int32_t* active, float cx, float cy, float cz, float radius) {
  require_mesh();
  require(active != nullptr, MGPBD_EINVAL, "active must be a device array of nt int32");
  launch_zone_proximity(t_i_, x_, nt_, cx, cy, cz, radius, active, stream_);
}

void Solver::zone_strain(int32_t* active, const float* x_old, float threshold, float dt) {
  require_mesh();
  require(active != nullptr, MGPBD_EINVAL, "active must be a device array of nt int32");
  require(dt > 0.0f, MGPBD_EINVAL, "dt must be positive");
  launch_zone_strain(t_i_, x_, x_old ? x_old : x_old_.p, nt_, threshold, dt, active, stream_);
}

void Solver::zone_expand(int32_t* active, int32_t n_rings) {
  require_mesh();
  require(active != nullptr && n_rings >= 0, MGPBD_EINVAL, "bad zone expansion arguments");
  if (!adj_ptr_.p) {
    std::vector<int32_t> t_host(4LL * nt_);
    MGPBD_CUDA(cudaMemcpyAsync(t_host.data(), t_i_, sizeof(int32_t) * t_host.size(),
                               cudaMemcpyDeviceToHost, stream_));
    MGPBD_CUDA(cudaStreamSynchronize(stream_));
    Csr a = face_adjacency(t_host.data(), nt_);
    upload(adj_ptr_, a.indptr, stream_);
    std::vector<int32_t> idx(a.indices);
    if (idx.empty()) idx.push_back(0);
    upload(adj_, idx, stream_);
    zone_scratch_.alloc(nt_);
  }
  launch_zone_expand(adj_ptr_.p, adj_.p, nt_, n_rings, active, zone_scratch_.p, stream_);
}

void Solver::mask_alpha(const int32_t* active, float* saved) {
  require_mesh();
  require(active != nullptr && saved != nullptr, MGPBD_EINVAL, "bad alpha mask arguments");
  launch_mask_alpha(active, alpha_.p, saved, nt_, stream_);
}

void Solver::restore_alpha(const float* saved) {
  require_mesh();
  require(saved != nullptr, MGPBD_EINVAL, "saved must be a device array of nt float");
  MGPBD_CUDA(cudaMemcpyAsync(alpha_.p, saved, sizeof(float) * nt_, cudaMemcpyDeviceToDevice,
                             stream_));
}

// one row-kernel pass over the library's CSR of `level`: op 0 y = A x,
// op 1 y = x + omega D^-1 (b - A x)
void Solver::level_sweep(int32_t level, int32_t op, const float* x, const float* b, float* y,
                         float omega) {
  require_init();
  require(level >= 0 && level < n_levels(), MGPBD_EINVAL, "level out of range");
  require(op == 0 || op == 1, MGPBD_EINVAL, "op must be 0 (spmv) or 1 (jacobi)");
  CsrView A = levels_[level].view();
  if (op == 0) launch_spmv(A, x, y, stream_);
  else launch_jacobi(A, b, x, y, omega, stream_);
}

JView Solver::jview() {
  JView j;
  j.nt = nt_;
  j.nv = nv_;
  j.t_i = t_i_;
  j.gradC = gradC_.p;
  j.gT = gT_.p;
  j.gV = gV_.p;
  j.inc_ptr = inc_ptr_.p;
  j.ne = inc_n_;
  j.invm = invm_;
  j.alpha = alpha_.p;
  j.dinv = jdinv_.p;
  j.unit_dinv = p_.cheb_scale == MGPBD_CHEB_UNSCALED;
  j.u = u_.p;
  j.n4 = n4_;
  j.gE = gE_.p;
  j.qE = reinterpret_cast<const int2*>(qE_.p);
  return j;
}

JVecs Solver::jvecs(const float* b, float* x) {
  JVecs v;
  v.b = b;
  v.x = x;
  v.xd = jxd_.p;
  v.r = jr_.p;
  v.z = jz_.p;
  v.d = jd_.p;
  v.p = jp_.p;
  v.ap = jap_.p;
  v.partials = partials_.p;
  return v;
}

// Per Newton iteration: vertex-major gradients, 1/diag(A) (all ones for the
// unscaled base), lambda_max of D^-1 A by 24 Lanczos steps (upper end taken 2% above the Ritz value; a
// Chebyshev interval that misses the top of the spectrum makes the
// preconditioner indefinite) and the Chebyshev coefficients.
void Solver::jform_setup(uint32_t* dev_status) {
  constexpr int kSteps = 24;
  JView j = jview();
  launch_jform_prepare(j, inc_ent_.p, gV_.p, jdinv_.p, gT_.p,
                       p_.cheb_scale == MGPBD_CHEB_UNSCALED, stream_);
  launch_jform_lanczos(j, pw_v_.p, jd_.p, pw_w_.p, partials_.p, jst_.p, kSteps, stream_);
  launch_cheb_coefficients(jst_.p, kSteps, p_.cheb_degree, p_.cheb_lo, dev_status, stream_);
  if (dev_status) return;  // captured: the status word is read after the graph
  sync_read(h_buf_, &jst_.p->cf.lmax, sizeof(double));
  if (!std::isfinite(h_buf_[0]) || !(h_buf_[0] > 0.0)) status_ |= MGPBD_STATUS_NAN;
}

// CG with the Chebyshev preconditioner as one CUDA graph: init, a device-side
// while loop over iterations (bounded by maxiter_cg on the device), and the
// float32 copy of the float64 solution.
int32_t Solver::pcg_cheb(const float* b, float* x) {
  cudaStream_t outer = stream_;
  if (p_.persistent) {
    int32_t its = 0, left = p_.maxiter_cg;
    bool warm = false;
    if (primal()) {
      // warm start: CG on the primal system to a loose dual residual (or
      // until it stalls), dlam = alpha~^-1 (b - J y) into x.  Declined when
      // the start's dual residual exceeds kPrimalMaxAmp |b|: measured on
      // stiff bodies, above ~1e6 the hand-over loses accuracy the float32
      // dual CG does not win back (1e-3 .. 1e-2 in dlam), below it the
      // solution matches a float64 direct solve to ~1e-5.
      constexpr int kPrimalStall = 16;
      constexpr double kPrimalMaxAmp = 1e6;
      PcgVecs v;
      v.b = b;
      v.dlam = x;
      v.y = pv_[0].p;
      v.yc = pv_[1].p;
      v.r = pv_[2].p;
      v.z = pv_[3].p;
      v.d = pv_[4].p;
      v.p = pv_[5].p;
      v.q = pv_[6].p;
      v.rhs = pv_[7].p;
      v.bi0 = pv_[8].p;
      v.bi1 = pv_[9].p;
      v.s = ps_.p;
      v.partials = partials_.p;
      v.partials_capacity = static_cast<int64_t>(kMaxReduceBlocks) * 16;
      v.gs = jgs_.p;
      const double tol = std::max<double>(p_.primal_tol, p_.rel_tol_cg);
      MGPBD_CUDA(cudaEventRecord(ev_[0], outer));
      launch_pcg_primal(jview(), v, pplan_, jpart_.p, cg_state_.p, p_.tol_cg, tol, p_.maxiter_cg,
                        p_.cheb_degree, p_.cheb_lo, kPrimalStall, kPrimalMaxAmp, barrier_limit_s_,
                        outer);
      MGPBD_CUDA(cudaEventRecord(ev_[1], outer));
      sync_read(h_state_, cg_state_.p, sizeof(CgState));
      stats_.ms_warm += event_ms(ev_[0], ev_[1]);
      stats_.cg_launches += 1;
      stats_.cg_iters_warm += h_state_->iters;
      const uint32_t st = static_cast<uint32_t>(h_state_->status);
      if (st & MGPBD_STATUS_SYNC_TIMEOUT) {
        status_ |= MGPBD_STATUS_SYNC_TIMEOUT;
        throw Error(MGPBD_ECUDA, "primal CG kernel: a grid barrier wait timed out");
      }
      // the dual solve below decides convergence; keep only the alarms
      status_ |= st & (MGPBD_STATUS_NAN | MGPBD_STATUS_PAP_NONPOS);
      if (st & MGPBD_STATUS_NAN) return h_state_->iters;
      its = h_state_->iters;
      left = p_.maxiter_cg - its;
      warm = h_state_->flags == 0;
      stats_.warm_amp = h_state_->rz_new;
      if (!warm) stats_.warm_declined += 1;
      if (left <= 0) {
        status_ |= MGPBD_STATUS_CG_MAXITER;
        return its;
      }
    }
    // one cooperative kernel for the (rest of the) solve; warm_substep: x
    // holds the previous substep's first solution
    if (warm_next_) warm = true;
    warm_next_ = false;
    return its + run_dual(b, x, p_.tol_cg, p_.rel_tol_cg, left, warm, ulo_.p);
  }
  if (!p_.use_graph) {
    // same kernels from the host; every kernel is a no-op once done is set
    JView j = jview();
    JVecs v = jvecs(b, x);
    launch_jcg_init(j, v, jst_.p, cg_state_.p, p_.tol_cg, p_.rel_tol_cg, p_.maxiter_cg, outer);
    launch_jcg_cheb_steps(j, v, jst_.p, cg_state_.p, p_.cheb_degree, true, outer);
    for (int32_t k = 0; k < p_.maxiter_cg; k += 8) {
      for (int c = 0; c < 8; ++c) launch_jcg_body(j, v, jst_.p, cg_state_.p, p_.cheb_degree, outer);
      sync_read(h_state_, cg_state_.p, sizeof(CgState));
      if (h_state_->done) break;
    }
    launch_jcg_finish(v, nt_, cg_state_.p, outer);
    sync_read(h_state_, cg_state_.p, sizeof(CgState));
    status_ |= static_cast<uint32_t>(h_state_->status);
    return h_state_->iters;
  }
  if (!jcg_exec_ || jcg_b_ != b || jcg_x_ != x) {
    if (jcg_exec_) {
      cudaGraphExecDestroy(jcg_exec_);
      jcg_exec_ = nullptr;
    }
    cudaStream_t cs, bs;
    MGPBD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    MGPBD_CUDA(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    try {
      JView j = jview();
      JVecs v = jvecs(b, x);
      long long c0 = g_launches.load();
      MGPBD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      launch_jcg_init(j, v, jst_.p, cg_state_.p, p_.tol_cg, p_.rel_tol_cg, p_.maxiter_cg, cs);
      launch_jcg_cheb_steps(j, v, jst_.p, cg_state_.p, p_.cheb_degree, true, cs);
      long long c1 = g_launches.load();
      cudaStreamCaptureStatus cst;
      const cudaGraphNode_t* deps = nullptr;
      size_t ndeps = 0;
      MGPBD_CUDA(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &graph, &deps, nullptr, &ndeps));
      cudaGraphConditionalHandle handle;
      MGPBD_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
      cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t cond;
      MGPBD_CUDA(cudaGraphAddNode(&cond, graph, deps, nullptr, ndeps, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      MGPBD_CUDA(cudaStreamUpdateCaptureDependencies(cs, &cond, nullptr, 1, cudaStreamSetCaptureDependencies));
      MGPBD_CUDA(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      launch_jcg_body(j, v, jst_.p, cg_state_.p, p_.cheb_degree, bs);
      k_set_cond<<<1, 1, 0, bs>>>(handle, cg_state_.p);
      MGPBD_CHECK_LAUNCH();
      long long c2 = g_launches.load();
      MGPBD_CUDA(cudaStreamEndCapture(bs, &body));
      launch_jcg_finish(v, nt_, cg_state_.p, cs);
      long long c3 = g_launches.load();
      g_launches.fetch_sub(c3 - c0);
      jgraph_init_launches_ = (c1 - c0) + (c3 - c2);
      jgraph_body_launches_ = c2 - c1;
      MGPBD_CUDA(cudaStreamEndCapture(cs, &graph));
      MGPBD_CUDA(cudaGraphInstantiate(&jcg_exec_, graph, 0));
      cudaGraphDestroy(graph);
    } catch (...) {
      cudaStreamCaptureStatus cst;
      if (cudaStreamIsCapturing(bs, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
        cudaGraph_t g2;
        cudaStreamEndCapture(bs, &g2);
      }
      if (cudaStreamIsCapturing(cs, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
        cudaGraph_t g2 = nullptr;
        cudaStreamEndCapture(cs, &g2);
        if (g2) cudaGraphDestroy(g2);
      }
      cudaGetLastError();
      cudaStreamDestroy(cs);
      cudaStreamDestroy(bs);
      throw;
    }
    cudaStreamDestroy(cs);
    cudaStreamDestroy(bs);
    jcg_b_ = b;
    jcg_x_ = x;
  }
  MGPBD_CUDA(cudaGraphLaunch(jcg_exec_, outer));
  sync_read(h_state_, cg_state_.p, sizeof(CgState));
  g_launches.fetch_add(jgraph_init_launches_ + jgraph_body_launches_ * h_state_->body_runs);
  status_ |= static_cast<uint32_t>(h_state_->status);
  return h_state_->iters;
}

// ---------------------------------------------------------------------------
void Solver::make_prediction() {
  require_mesh();
  launch_predict(x_, v_, x_old_.p, x_pred_.p, invm_, nv_, p_.dt, p_.gravity, p_.damp,
                 p_.kinematic_pins, stream_);
}

void Solver::update_vel() {
  require_mesh();
  launch_update_vel(x_, x_old_.p, v_, nv_, p_.dt, p_.damp, stream_);
}

void Solver::step(int32_t frame) {
  make_prediction();
  solve(frame);
  update_vel();
}

void Solver::compute_constraints() {
  require_mesh();
  launch_constraints(x_, t_i_, ctype_.p, dm_inv_.p, rest_vol_.p, nt_, C_.p, gradC_.p, stream_);
}

// _fill_A_and_update_gpu (cons/mgpbd_gpu.py:320-324)
void Solver::fill_matrices() {
  require_mesh();
  if (cheb()) {
    // matrix-free: no CSR values; the gradients are the operator
    jform_setup();
    return;
  }
  cudaStream_t s = stream_;
  Level& L0 = levels_[0];
  launch_fill_A(L0.indptr.p, L0.indices.p, t_i_, invm_, gradC_.p, alpha_.p, nt_, L0.data.p,
                L0.diag_inv.p, s);
  refill_coarse();
}

// update_all_coarse_matrices (cons/mgpcg_gpu.py:200-212) from the current
// level-0 values, then the per-level smoother weights and coarse factor.
void Solver::refill_coarse() {
  require_init();
  cudaStream_t s = stream_;
  for (size_t l = 1; l < levels_.size(); ++l) {
    Level& C = levels_[l];
    launch_rap_refill(C.contrib_off.p, C.contrib_idx.p, levels_[l - 1].data.p, C.nnz, C.data.p, s);
    launch_diag_inv_pos(C.diag_pos.p, C.data.p, C.n, C.diag_inv.p, s);
  }
  if (p_.smoother == MGPBD_SMOOTH_JACOBI_SAFE) update_smoother_weights();
  if (p_.coarse_solver == MGPBD_COARSE_DENSE_F64) factor_coarsest();
}

void Solver::update_smoother_weights() {
  cudaStream_t s = stream_;
  int32_t nmax = static_cast<int32_t>(pw_b_.n);
  int64_t off = 0;
  for (Level& L : levels_) {
    int blocks = std::min(kMaxReduceBlocks, std::max(1, ceil_div(L.n, 256)));
    float* a = pw_a_.p + off;
    for (int it = 0; it < 6; ++it) {
      k_pw_step<<<blocks, 256, 0, s>>>(L.n, L.indptr.p, L.indices.p, L.data.p, L.diag_inv.p, a,
                                       pw_b_.p, partials_.p);
      MGPBD_CHECK_LAUNCH();
      launch_finalize(partials_.p, blocks, 1, scalars_.p + 8, s);
      MGPBD_CUDA(cudaMemcpyAsync(a, pw_b_.p, sizeof(float) * L.n, cudaMemcpyDeviceToDevice, s));
      k_pw_scale<<<blocks, 256, 0, s>>>(a, L.n, scalars_.p + 8);
      MGPBD_CHECK_LAUNCH();
    }
    k_pw_weight<<<1, 1, 0, s>>>(scalars_.p + 8, p_.omega_jacobi, L.omega.p);
    MGPBD_CHECK_LAUNCH();
    off += nmax;
  }
}

void Solver::factor_coarsest() {
  Level& L = levels_.back();
  launch_dense_chol_factor(L.view(), chol_.p, L.n, chol_info_.p, stream_);
}

double Solver::compute_rhs() {
  require_mesh();
  int blocks = reduce_blocks(nt_);
  launch_rhs(C_.p, alpha_.p, lambda_.p, nt_, rhs_.p, partials_.p, stream_);
  return std::sqrt(finalize_read(partials_.p, blocks));
}

// ---------------------------------------------------------------------------
// Jacobi sweeps on level l (cons/sparse_gpu.py:134-144 + gpu_copy); cur holds
// the iterate, nxt the scratch, and they swap after each sweep.
void Solver::smooth_level(int32_t l, const float* b, float*& cur, float*& nxt, int sweeps,
                          bool from_zero, const CgState* guard) {
  Level& L = levels_[l];
  CsrView A = L.view();
  for (int it = 0; it < sweeps; ++it) {
    bool zero = from_zero && it == 0 && p_.mode == MGPBD_MODE_FAST;
    if (from_zero && it == 0 && !zero)
      MGPBD_CUDA(cudaMemsetAsync(cur, 0, sizeof(float) * L.n, stream_));
    launch_jacobi_gw(guard, A, b, zero ? nullptr : cur, nxt, p_.omega_jacobi, L.omega.p, stream_);
    std::swap(cur, nxt);
  }
  if (sweeps == 0 && from_zero) MGPBD_CUDA(cudaMemsetAsync(cur, 0, sizeof(float) * L.n, stream_));
}

// GPUMultigridSolver.vcycle (cons/mgpcg_gpu.py:214-259) with a zero initial
// guess; the result ends in levels_[l].xa.
void Solver::vcycle(int32_t l, const float* b, const CgState* guard) {
  Level& L = levels_[l];
  float* cur = L.xa.p;
  float* nxt = L.xb.p;
  if (l == n_levels() - 1) {
    if (p_.coarse_solver == MGPBD_COARSE_DENSE_F64) {
      launch_dense_chol_solve(guard, chol_.p, L.n, b, L.xa.p, stream_);
      return;
    }
    int sweeps = p_.coarse_sweeps > 0 ? p_.coarse_sweeps : std::min(50, L.n);
    smooth_level(l, b, cur, nxt, sweeps, true, guard);
  } else {
    smooth_level(l, b, cur, nxt, p_.n_smooth, true, guard);
    Level& C = levels_[l + 1];
    // with cg_alias the level-0 residual lands in the CG residual vector, as
    // in the reference (cons/mgpcg_gpu.py:239-240 with :275)
    float* res = (l == 0 && p_.cg_alias) ? cg_r_.p : L.r.p;
    launch_residual_g(guard, L.view(), b, cur, res, stream_);
    launch_restrict_g(guard, L.mem_ptr.p, L.mem_rows.p, res, C.n, C.b.p, stream_);
    if (l == 0)
      coarse_correction(guard);
    else
      vcycle(l + 1, C.b.p, guard);
    launch_prolong_add_g(guard, L.agg.p, C.xa.p, L.n, cur, stream_);
    smooth_level(l, b, cur, nxt, p_.n_smooth, false, guard);
  }
  if (cur != L.xa.p)
    MGPBD_CUDA(cudaMemcpyAsync(L.xa.p, cur, sizeof(float) * L.n, cudaMemcpyDeviceToDevice, stream_));
}

// The coarse correction of the level-0 V-cycle: the recursion (the
// reference's), the learned weights, or -- on the first V-cycle of a learned
// solve -- both, the plain one judging the learned one by coarse energy.
void Solver::coarse_correction(const CgState* guard) {
  Level& C = levels_[1];
  cudaStream_t s = stream_;
  if (judge_pending_) {
    judge_pending_ = false;
    apply_coarse_weights(C.n, net_w_.p, C.diag_inv.p, C.b.p, net_e_.p, s);
    vcycle(1, C.b.p, guard);
    double el = coarse_energy(net_e_.p, C.b.p);
    double ep = coarse_energy(C.xa.p, C.b.p);
    stats_.coarse_energy_learned += el;
    stats_.coarse_energy_plain += ep;
    net_active_ = std::isfinite(el) && el <= static_cast<double>(p_.learned_accept) * ep;
    if (net_active_)
      MGPBD_CUDA(cudaMemcpyAsync(C.xa.p, net_e_.p, sizeof(float) * C.n, cudaMemcpyDeviceToDevice, s));
    else
      stats_.learned_rejected += 1;
    return;
  }
  if (net_active_) {
    apply_coarse_weights(C.n, net_w_.p, C.diag_inv.p, C.b.p, C.xa.p, s);
    return;
  }
  vcycle(1, C.b.p, guard);
  if (rec_count_ < rec_cap_) {
    if (rec_calls_ % rec_every_ == 0) {
      const int64_t off = static_cast<int64_t>(rec_count_) * C.n;
      MGPBD_CUDA(cudaMemcpyAsync(rec_rc_ + off, C.b.p, sizeof(float) * C.n, cudaMemcpyDeviceToDevice, s));
      MGPBD_CUDA(cudaMemcpyAsync(rec_ec_ + off, C.xa.p, sizeof(float) * C.n, cudaMemcpyDeviceToDevice, s));
      ++rec_count_;
    }
    ++rec_calls_;
  }
}

void Solver::autotune_rows(int32_t reps, int32_t* codes, float* us) {
  require_init();
  for (int32_t l = 0; l < n_levels(); ++l) {
    Level& L = levels_[l];
    MGPBD_CUDA(cudaMemsetAsync(L.xa.p, 0, sizeof(float) * L.n, stream_));
    MGPBD_CUDA(cudaMemsetAsync(L.b.p, 0, sizeof(float) * L.n, stream_));
    float t = 0.f;
    CsrView v = L.view();
    L.shape = tune_row_shape(v, L.xa.p, L.b.p, L.xb.p, reps, stream_, &t);
    if (codes) codes[l] = row_shape_code(L.shape);
    if (us) us[l] = t;
  }
  // a captured CG loop holds the old shapes
  if (cg_exec_) {
    cudaGraphExecDestroy(cg_exec_);
    cg_exec_ = nullptr;
    cg_graph_b_ = nullptr;
    cg_graph_x_ = nullptr;
  }
}

int32_t Solver::level_row_shape(int32_t l) const {
  const Level& L = level(l);
  return L.shape < 0 ? 0 : row_shape_code(L.shape);
}

void Solver::set_level_row_shape(int32_t l, int32_t code) {
  require_init();
  require(l >= 0 && l < n_levels(), MGPBD_EINVAL, "level out of range");
  levels_[l].shape = code == 0 ? -1 : row_shape_index(code);
  if (cg_exec_) {
    cudaGraphExecDestroy(cg_exec_);
    cg_exec_ = nullptr;
    cg_graph_b_ = nullptr;
    cg_graph_x_ = nullptr;
  }
}

NetGraph Solver::net_graph() const {
  const Level& C = levels_[1];
  NetGraph g;
  g.n = C.n;
  g.nnz = C.nnz;
  g.indptr = C.indptr.p;
  g.indices = C.indices.p;
  g.data = C.data.p;
  g.diag_inv = C.diag_inv.p;
  return g;
}

double Solver::coarse_energy(const float* e, const float* r) {
  Level& C = levels_[1];
  cudaStream_t s = stream_;
  int blocks = reduce_blocks(C.n);
  launch_spmv(C.view(), e, net_t_.p, s);
  launch_dot_partials(e, net_t_.p, C.n, partials_.p, s);
  launch_dot_partials(e, r, C.n, partials_.p + blocks, s);
  launch_finalize(partials_.p, blocks, 2, scalars_.p + 48, s);
  sync_read(h_buf_ + 48, scalars_.p + 48, 2 * sizeof(double));
  return 0.5 * h_buf_[48] - h_buf_[49];
}

void Solver::record_coarse(float* rc, float* ec, int32_t capacity, int32_t every) {
  require_init();
  require(n_levels() >= 2, MGPBD_ESTATE, "record_coarse: the hierarchy has one level");
  require(capacity >= 0 && every >= 1, MGPBD_EINVAL, "record_coarse: capacity < 0 or every < 1");
  require(capacity == 0 || (rc && ec), MGPBD_EINVAL, "record_coarse: null buffer");
  rec_rc_ = rc;
  rec_ec_ = ec;
  rec_cap_ = capacity;
  rec_every_ = every;
  rec_count_ = 0;
  rec_calls_ = 0;
}

void Solver::precondition(const CgState* guard) {
  const float* b0 = cg_r_.p;
  if (p_.cg_alias && n_levels() > 1) {
    // the reference copies r into _b[0] before vcycle(0) (cons/mgpcg_gpu.py:278,311)
    MGPBD_CUDA(cudaMemcpyAsync(levels_[0].b.p, cg_r_.p, sizeof(float) * nt_,
                               cudaMemcpyDeviceToDevice, stream_));
    b0 = levels_[0].b.p;
  }
  vcycle(0, b0, guard);
}

void Solver::vcycle_into(const float* r, float* z) {
  require_init();
  require(!cheb(), MGPBD_ENOTSUP, "no V-cycle: the solver uses the Chebyshev preconditioner");
  vcycle(0, r, nullptr);
  MGPBD_CUDA(cudaMemcpyAsync(z, levels_[0].xa.p, sizeof(float) * nt_, cudaMemcpyDeviceToDevice,
                             stream_));
}

// One CG iteration (cons/mgpcg_gpu.py:289-327) on device scalars.
void Solver::cg_body(const float* b, float* x) {
  (void)b;
  cudaStream_t s = stream_;
  CgState* st = cg_state_.p;
  int64_t n = nt_;
  int blocks = reduce_blocks(n);
  launch_spmv_dot_g(st, levels_[0].view(), cg_p_.p, cg_ap_.p, partials_.p, s);
  launch_cg_alpha(st, partials_.p, blocks, s);
  launch_cg_update_xr(st, cg_p_.p, cg_ap_.p, x, cg_r_.p, n, partials_.p, s);
  launch_cg_check(st, partials_.p, blocks, s);
  precondition(st);
  launch_dot_partials_g(st, cg_r_.p, levels_[0].xa.p, n, partials_.p, s);
  launch_cg_beta(st, partials_.p, blocks, s);
  launch_cg_update_p(st, levels_[0].xa.p, cg_p_.p, n, s);
}

// PCG with the learned coarse correction (MGPBD_PRECOND_LEARNED): the
// iterations of pcg(), with the network's weights computed once for the
// solve, the judge on the first V-cycle and a restart from the current
// iterate when the learned preconditioner stalls (the preconditioner is
// linear and fixed between restarts, so standard CG applies).
int32_t Solver::pcg_learned(const float* b, float* x) {
  require(net_ != nullptr, MGPBD_ESTATE,
          "MGPBD_PRECOND_LEARNED: no coarse network attached (mgpbd_set_coarse_net)");
  require(n_levels() >= 2, MGPBD_ESTATE, "MGPBD_PRECOND_LEARNED needs a level-1 aggregate graph");
  require(!p_.cg_alias, MGPBD_ENOTSUP, "MGPBD_PRECOND_LEARNED does not combine with cg_alias");
  cudaStream_t s = stream_;
  int64_t n = nt_;
  int blocks = reduce_blocks(n);
  const int32_t n1 = levels_[1].n;
  if (net_e_.n < n1) {
    net_e_.alloc(n1);
    net_t_.alloc(n1);
    net_w_.alloc(n1);
  }
  // the network's weights for this solve's level-1 matrix
  net_->weights(net_graph(), net_w_.p, s);
  const size_t vb = sizeof(float) * n;
  float* z = levels_[0].xa.p;
  MGPBD_CUDA(cudaMemsetAsync(x, 0, vb, s));
  MGPBD_CUDA(cudaMemcpyAsync(cg_r_.p, b, vb, cudaMemcpyDeviceToDevice, s));
  judge_pending_ = true;
  precondition(nullptr);
  judge_pending_ = false;
  MGPBD_CUDA(cudaMemcpyAsync(cg_p_.p, z, vb, cudaMemcpyDeviceToDevice, s));
  MGPBD_CUDA(cudaMemcpyAsync(cg_z_.p, z, vb, cudaMemcpyDeviceToDevice, s));
  launch_dot_partials(cg_r_.p, z, n, partials_.p, s);
  launch_dot_partials(b, b, n, partials_.p + blocks, s);
  launch_cg_init(cg_state_.p, partials_.p, blocks, p_.tol_cg, p_.rel_tol_cg, p_.maxiter_cg, s);
  double best = std::numeric_limits<double>::infinity();
  int32_t best_at = 0;
  const uint32_t broken = MGPBD_STATUS_NAN | MGPBD_STATUS_PAP_NONPOS;
  for (int32_t k = 0; k < p_.maxiter_cg; ++k) {
    cg_body(b, x);
    sync_read(h_state_, cg_state_.p, sizeof(CgState));
    const bool bad = net_active_ && (static_cast<uint32_t>(h_state_->status) & broken);
    if (h_state_->done && !bad) break;
    if (!net_active_) continue;
    if (h_state_->rr < best) {
      best = h_state_->rr;
      best_at = h_state_->iters;
    }
    if (bad || (p_.learned_stall > 0 && h_state_->iters - best_at >= p_.learned_stall)) {
      // fall back to the plain V-cycle from the current iterate
      net_active_ = false;
      stats_.learned_fallbacks += 1;
      if (static_cast<uint32_t>(h_state_->status) & MGPBD_STATUS_NAN) {
        MGPBD_CUDA(cudaMemsetAsync(x, 0, vb, s));
        MGPBD_CUDA(cudaMemcpyAsync(cg_r_.p, b, vb, cudaMemcpyDeviceToDevice, s));
      } else {
        launch_residual(levels_[0].view(), b, x, cg_r_.p, s);
      }
      precondition(nullptr);
      MGPBD_CUDA(cudaMemcpyAsync(cg_p_.p, z, vb, cudaMemcpyDeviceToDevice, s));
      MGPBD_CUDA(cudaMemcpyAsync(cg_z_.p, z, vb, cudaMemcpyDeviceToDevice, s));
      launch_dot_partials(cg_r_.p, z, n, partials_.p, s);
      launch_cg_restart(cg_state_.p, partials_.p, blocks, static_cast<int32_t>(broken), s);
      sync_read(h_state_, cg_state_.p, sizeof(CgState));
      if (h_state_->done) break;
    }
  }
  sync_read(h_state_, cg_state_.p, sizeof(CgState));
  if (net_active_) stats_.learned_solves += 1;
  net_active_ = false;
  status_ |= static_cast<uint32_t>(h_state_->status);
  return h_state_->iters;
}

// GPUMultigridSolver.solve (cons/mgpcg_gpu.py:261-329)
int32_t Solver::pcg(const float* b, float* x) {
  require_init();
  dual_x_ = nullptr;
  if (cheb()) return pcg_cheb(b, x);
  if (learned()) return pcg_learned(b, x);
  if (p_.mode == MGPBD_MODE_FAST && p_.use_graph && b == rhs_.p && x == dlam_.p &&
      rec_count_ >= rec_cap_)
    return pcg_graph(b, x);
  cudaStream_t s = stream_;
  int64_t n = nt_;
  int blocks = reduce_blocks(n);
  MGPBD_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * n, s));
  MGPBD_CUDA(cudaMemcpyAsync(cg_r_.p, b, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  precondition(nullptr);
  MGPBD_CUDA(cudaMemcpyAsync(cg_p_.p, levels_[0].xa.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  launch_dot_partials(cg_r_.p, levels_[0].xa.p, n, partials_.p, s);
  launch_dot_partials(b, b, n, partials_.p + blocks, s);
  launch_cg_init(cg_state_.p, partials_.p, blocks, p_.tol_cg, p_.rel_tol_cg, p_.maxiter_cg, s);
  for (int32_t k = 0; k < p_.maxiter_cg; ++k) {
    cg_body(b, x);
    sync_read(h_state_, cg_state_.p, sizeof(CgState));
    if (h_state_->done) break;
  }
  sync_read(h_state_, cg_state_.p, sizeof(CgState));
  status_ |= static_cast<uint32_t>(h_state_->status);
  return h_state_->iters;
}

// FAST mode: the whole CG loop is one CUDA graph whose iterations run under a
// device-side while condition (no host round trip per iteration).  The loop
// is bounded on the device by maxiter_cg (k_cg_beta sets done).
int32_t Solver::pcg_graph(const float* b, float* x) {
  cudaStream_t outer = stream_;
  if (!cg_exec_ || cg_graph_b_ != b || cg_graph_x_ != x) {
    if (cg_exec_) {
      cudaGraphExecDestroy(cg_exec_);
      cg_exec_ = nullptr;
    }
    cudaStream_t cs, bs;
    MGPBD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    MGPBD_CUDA(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    try {
      int64_t n = nt_;
      int blocks = reduce_blocks(n);
      long long c0 = g_launches.load();
      MGPBD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      stream_ = cs;
      MGPBD_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * n, cs));
      MGPBD_CUDA(cudaMemcpyAsync(cg_r_.p, b, sizeof(float) * n, cudaMemcpyDeviceToDevice, cs));
      precondition(nullptr);
      MGPBD_CUDA(cudaMemcpyAsync(cg_p_.p, levels_[0].xa.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, cs));
      launch_dot_partials(cg_r_.p, levels_[0].xa.p, n, partials_.p, cs);
      launch_dot_partials(b, b, n, partials_.p + blocks, cs);
      launch_cg_init(cg_state_.p, partials_.p, blocks, p_.tol_cg, p_.rel_tol_cg, p_.maxiter_cg, cs);
      long long c1 = g_launches.load();
      cudaStreamCaptureStatus cst;
      const cudaGraphNode_t* deps = nullptr;
      size_t ndeps = 0;
      MGPBD_CUDA(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &graph, &deps, nullptr, &ndeps));
      cudaGraphConditionalHandle handle;
      MGPBD_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
      cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t cond;
      MGPBD_CUDA(cudaGraphAddNode(&cond, graph, deps, nullptr, ndeps, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      MGPBD_CUDA(cudaStreamUpdateCaptureDependencies(cs, &cond, nullptr, 1, cudaStreamSetCaptureDependencies));
      MGPBD_CUDA(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      stream_ = bs;
      cg_body(b, x);
      k_set_cond<<<1, 1, 0, bs>>>(handle, cg_state_.p);
      MGPBD_CHECK_LAUNCH();
      long long c2 = g_launches.load();
      // captured launches run later, when the graph does
      g_launches.fetch_sub(c2 - c0);
      graph_init_launches_ = c1 - c0;
      graph_body_launches_ = c2 - c1;
      MGPBD_CUDA(cudaStreamEndCapture(bs, &body));
      stream_ = outer;
      MGPBD_CUDA(cudaStreamEndCapture(cs, &graph));
      MGPBD_CUDA(cudaGraphInstantiate(&cg_exec_, graph, 0));
      cudaGraphDestroy(graph);
    } catch (...) {
      stream_ = outer;
      cudaStreamCaptureStatus cst;
      if (cudaStreamIsCapturing(bs, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
        cudaGraph_t g2;
        cudaStreamEndCapture(bs, &g2);
      }
      if (cudaStreamIsCapturing(cs, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
        cudaGraph_t g2 = nullptr;
        cudaStreamEndCapture(cs, &g2);
        if (g2) cudaGraphDestroy(g2);
      }
      cudaGetLastError();
      cudaStreamDestroy(cs);
      cudaStreamDestroy(bs);
      throw;
    }
    cudaStreamDestroy(cs);
    cudaStreamDestroy(bs);
    cg_graph_b_ = b;
    cg_graph_x_ = x;
  }
  MGPBD_CUDA(cudaGraphLaunch(cg_exec_, outer));
  sync_read(h_state_, cg_state_.p, sizeof(CgState));
  g_launches.fetch_add(graph_init_launches_ + graph_body_launches_ * h_state_->body_runs);
  status_ |= static_cast<uint32_t>(h_state_->status);
  return h_state_->iters;
}

// _zero_dpos + _scatter_dlam_gpu (cons/mgpbd_gpu.py:330-355)
void Solver::scatter(const float* dlam) {
  require_mesh();
  launch_lambda_update(lambda_.p, dlam, nt_, stream_);
  // after a persistent dual solve into this dlam, its low part (jxc_) joins
  // a float64 scatter
  const float* lo = (dual_x_ != nullptr && dual_x_ == dlam) ? jxc_.p : nullptr;
  launch_scatter(inc_ptr_.p, inc_ent_.p, invm_, dlam, gradC_.p, dpos_.p, nv_, stream_, lo);
}

// _line_search (cons/mgpbd_gpu.py:379-391): backtracking from omega = 1 by
// halves, at most 10 trials, accept the first trial whose dual residual is
// below the one at the current positions (with the updated lambda).  The
// current norm reuses C of this Newton iteration (same positions, same
// arithmetic as recomputing it); trials 2..10 are evaluated in one pass
// only when trial 1 fails.
double Solver::line_search() {
  require_mesh();
  cudaStream_t s = stream_;
  int blocks = reduce_blocks(nt_);
  h_buf_[0] = 1.0;
  MGPBD_CUDA(cudaMemcpyAsync(omegas_.p, h_buf_, sizeof(double), cudaMemcpyHostToDevice, s));
  launch_dual_sq(C_.p, alpha_.p, lambda_.p, nt_, partials_.p, s);
  launch_dual_trial(x_, dpos_.p, omegas_.p, 1, t_i_, ctype_.p, dm_inv_.p, rest_vol_.p, alpha_.p, lambda_.p, nt_,
                    partials_.p + blocks, s);
  launch_finalize(partials_.p, blocks, 2, scalars_.p, s);
  sync_read(h_buf_, scalars_.p, 2 * sizeof(double));
  double current = std::sqrt(h_buf_[0]);
  double trial = std::sqrt(h_buf_[1]);
  if (trial < current) return 1.0;
  double om[9];
  for (int k = 0; k < 9; ++k) om[k] = std::ldexp(1.0, -(k + 1));
  std::memcpy(h_buf_, om, sizeof(om));
  MGPBD_CUDA(cudaMemcpyAsync(omegas_.p, h_buf_, sizeof(om), cudaMemcpyHostToDevice, s));
  launch_dual_trial(x_, dpos_.p, omegas_.p, 9, t_i_, ctype_.p, dm_inv_.p, rest_vol_.p, alpha_.p, lambda_.p, nt_,
                    partials_.p, s);
  launch_finalize(partials_.p, blocks, 9, scalars_.p, s);
  sync_read(h_buf_, scalars_.p, 9 * sizeof(double));
  for (int k = 0; k < 9; ++k)
    if (std::sqrt(h_buf_[k]) < current) return om[k];
  return std::ldexp(1.0, -10);
}

void Solver::apply_dpos(double omega) {
  require_mesh();
  launch_apply(x_, dpos_.p, invm_, nv_, static_cast<float>(omega), stream_);
}

// MGPBDSolverGPU.solve (cons/mgpbd_gpu.py:397-446)
void Solver::solve(int32_t frame) {
  (void)frame;
  require_mesh();
  if (nb_ > 0) {
    if (p_.use_graph) solve_bodies_graph();
    else solve_bodies();
    return;
  }
  status_ = 0;
  MGPBD_CUDA(cudaMemsetAsync(lambda_.p, 0, sizeof(float) * nt_, stream_));
  double r0 = 0.0;
  stats_.newton_iters = 0;
  stats_.cg_iters_total = 0;
  stats_.cg_iters_last = 0;
  stats_.omega_last = 1.0;
  stats_.cg_iters_warm = 0;
  stats_.cg_launches = 0;
  stats_.ms_warm = 0.0;
  stats_.ms_dual = 0.0;
  stats_.warm_amp = 0.0;
  stats_.warm_declined = 0;
  stats_.learned_fallbacks = 0;
  stats_.learned_rejected = 0;
  stats_.learned_solves = 0;
  stats_.coarse_energy_learned = 0.0;
  stats_.coarse_energy_plain = 0.0;
  log_.clear();
  auto now = [] {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  };
  for (int32_t ite = 0; ite < p_.maxiter; ++ite) {
    compute_constraints();
    double r = compute_rhs();
    if (ite == 0) {
      r0 = r;
      stats_.residual0 = r;
    }
    stats_.residual = r;
    if (!std::isfinite(r)) {
      status_ |= MGPBD_STATUS_NAN;
      break;
    }
    if (r < p_.atol || (r0 > 1e-12 && r < p_.rtol * r0)) {
      log_.push_back({double(ite), r, 0.0, 1.0, now()});
      break;
    }
    fill_matrices();
    const bool warm_sub = ite == 0 && p_.warm_substep && cheb() && p_.persistent && !primal() &&
                          p_.mode == MGPBD_MODE_FAST;
    if (warm_sub && have_prev_) {
      MGPBD_CUDA(cudaMemcpyAsync(dlam_.p, dlam_prev_.p, sizeof(float) * nt_,
                                 cudaMemcpyDeviceToDevice, stream_));
      warm_next_ = true;
    }
    int32_t it = pcg(rhs_.p, dlam_.p);
    warm_next_ = false;
    if (warm_sub && !(status_ & (MGPBD_STATUS_NAN | MGPBD_STATUS_CG_MAXITER))) {
      if (dlam_prev_.n != nt_) dlam_prev_.alloc(nt_);
      MGPBD_CUDA(cudaMemcpyAsync(dlam_prev_.p, dlam_.p, sizeof(float) * nt_,
                                 cudaMemcpyDeviceToDevice, stream_));
      have_prev_ = true;
    }
    scatter(dlam_.p);
    double omega = p_.use_line_search ? line_search() : 1.0;
    apply_dpos(omega);
    log_.push_back({double(ite), r, double(it), omega, now()});
    stats_.newton_iters = ite + 1;
    stats_.cg_iters_total += it;
    stats_.cg_iters_last = it;
    stats_.omega_last = omega;
    if (ite + 1 == p_.maxiter) status_ |= MGPBD_STATUS_NEWTON_MAXITER;
  }
  stats_.status = status_;
}

// One cooperative dual CG kernel from x (warm) or 0 to |r| <= max(tol_abs,
// tol_rel |b|) or maxit iterations; returns its iterations.
int32_t Solver::run_dual(const float* b, float* x, double tol_abs, double tol_rel, int32_t maxit,
                         bool warm, float4* ulo) {
  cudaStream_t outer = stream_;
  JcgVecs v = dual_vecs(b, x);
  v.ulo = ulo;
  MGPBD_CUDA(cudaEventRecord(ev_[0], outer));
  dual_x_ = nullptr;
  launch_jcg_persistent(jview(), v, jplan_, jpart_.p, jst_.p, cg_state_.p, tol_abs, tol_rel, maxit,
                        p_.cheb_degree, warm, barrier_limit_s_, outer);
  dual_x_ = x;
  MGPBD_CUDA(cudaEventRecord(ev_[1], outer));
  sync_read(h_state_, cg_state_.p, sizeof(CgState));
  stats_.ms_dual += event_ms(ev_[0], ev_[1]);
  stats_.cg_launches += 1;
  if (static_cast<uint32_t>(h_state_->status) & MGPBD_STATUS_SYNC_TIMEOUT) {
    status_ |= MGPBD_STATUS_SYNC_TIMEOUT;
    throw Error(MGPBD_ECUDA, "persistent CG kernel: a grid barrier wait timed out");
  }
  status_ |= static_cast<uint32_t>(h_state_->status);
  return h_state_->iters;
}

// ---------------------------------------------------------------------------
// Packed independent bodies

namespace {
constexpr int32_t kBodyChunk = 4096;  // constraints per reduction chunk
constexpr int32_t kCgChunk = 256;     // constraints per chunk of the per-body CG
constexpr int kBodyTrials = 10;       // line-search steps 1, 1/2, ..., 1/512
}  // namespace

void Solver::set_bodies(int32_t n_bodies, const int32_t* vert_off, int32_t n_segs,
                        const int32_t* segs) {
  require(x_ && t_i_ && !matrix_mode_, MGPBD_ESTATE, "mgpbd_set_mesh must come before mgpbd_set_bodies");
  if (n_bodies == 0) {
    nb_ = 0;
    inited_ = false;
    return;
  }
  require(n_bodies > 0 && vert_off && segs && n_segs >= n_bodies, MGPBD_EINVAL,
          "bodies: null array or fewer constraint ranges than bodies");
  require(vert_off[0] == 0 && vert_off[n_bodies] == nv_, MGPBD_EINVAL,
          "bodies: vert_off must run from 0 to nv");
  for (int32_t b = 0; b < n_bodies; ++b)
    require(vert_off[b + 1] > vert_off[b], MGPBD_EINVAL, "bodies: every body needs vertices");
  std::vector<uint8_t> seen(n_bodies, 0);
  int32_t at = 0;
  for (int32_t k = 0; k < n_segs; ++k) {
    const int32_t lo = segs[3 * k], hi = segs[3 * k + 1], body = segs[3 * k + 2];
    require(lo == at && hi > lo && hi <= nt_, MGPBD_EINVAL,
            "bodies: constraint ranges must cover [0, nt) in order, each non-empty");
    require(body >= 0 && body < n_bodies, MGPBD_EINVAL, "bodies: body id out of range");
    seen[body] = 1;
    at = hi;
  }
  require(at == nt_, MGPBD_EINVAL, "bodies: constraint ranges must end at nt");
  for (uint8_t u : seen) require(u != 0, MGPBD_EINVAL, "bodies: a body without constraints");
  nb_ = n_bodies;
  body_vert_off_.assign(vert_off, vert_off + n_bodies + 1);
  body_segs_.assign(segs, segs + 3LL * n_segs);
  inited_ = false;
}

void Solver::init_bodies(const std::vector<int32_t>& t_host) {
  require(cheb() && p_.persistent && p_.mode == MGPBD_MODE_FAST, MGPBD_ENOTSUP,
          "packed bodies run the FAST persistent Chebyshev CG (mode fast, precond cheb)");
  cudaStream_t s = stream_;
  std::vector<int32_t> cb(nt_), vb(nv_), ch;
  chunk_body_.clear();
  for (size_t k = 0; k < body_segs_.size(); k += 3) {
    const int32_t lo = body_segs_[k], hi = body_segs_[k + 1], body = body_segs_[k + 2];
    for (int32_t t = lo; t < hi; ++t) cb[t] = body;
    for (int32_t c = lo; c < hi; c += kBodyChunk) {
      ch.push_back(c);
      ch.push_back(std::min(hi, c + kBodyChunk));
      chunk_body_.push_back(body);
    }
  }
  for (int32_t b = 0; b < nb_; ++b)
    for (int32_t v = body_vert_off_[b]; v < body_vert_off_[b + 1]; ++v) vb[v] = b;
  // a constraint may only touch its own body's vertices (the bodies are
  // independent: block-diagonal A)
  for (int32_t t = 0; t < nt_; ++t)
    for (int l = 0; l < 4; ++l)
      require(vb[t_host[4LL * t + l]] == cb[t], MGPBD_EINVAL,
              "bodies: a constraint touches another body's vertices");
  upload(chunks_, ch, s);
  upload(cons_body_, cb, s);
  upload(vert_body_, vb, s);
  body_active_.alloc(nb_);
  body_omega_.alloc(nb_);
  chunk_partials_.alloc(static_cast<int64_t>(kBodyTrials) * static_cast<int64_t>(chunk_body_.size()));
  body_newton_.assign(nb_, 0);
  body_r0_.assign(nb_, 0.0);
  body_r_.assign(nb_, 0.0);
  body_omega_h_.assign(nb_, 1.0);
  // each body's chunks in ascending order (the host loop's summation order)
  std::vector<int32_t> cp(nb_ + 1, 0), ci(chunk_body_.size());
  for (int32_t b : chunk_body_) cp[b + 1]++;
  for (int32_t b = 0; b < nb_; ++b) cp[b + 1] += cp[b];
  {
    std::vector<int32_t> cur(cp.begin(), cp.end() - 1);
    for (size_t c = 0; c < chunk_body_.size(); ++c) ci[cur[chunk_body_[c]]++] = static_cast<int32_t>(c);
  }
  upload(body_chunk_ptr_, cp, s);
  upload(body_chunk_idx_, ci, s);
  // the per-body CG's chunks (at most kCgChunk constraints, inside one body)
  // and each body's chunk list
  {
    std::vector<int32_t> gch, gchb, gp(nb_ + 1, 0), gi;
    for (size_t k = 0; k < body_segs_.size(); k += 3) {
      const int32_t lo = body_segs_[k], hi = body_segs_[k + 1], body = body_segs_[k + 2];
      for (int32_t c = lo; c < hi; c += kCgChunk) {
        gch.push_back(c);
        gch.push_back(std::min(hi, c + kCgChunk));
        gchb.push_back(body);
      }
    }
    for (int32_t b : gchb) gp[b + 1]++;
    for (int32_t b = 0; b < nb_; ++b) gp[b + 1] += gp[b];
    gi.resize(gchb.size());
    std::vector<int32_t> cur(gp.begin(), gp.end() - 1);
    for (size_t c = 0; c < gchb.size(); ++c) gi[cur[gchb[c]]++] = static_cast<int32_t>(c);
    upload(bcg_ch_, gch, s);
    upload(bcg_chb_, gchb, s);
    upload(bcg_bptr_, gp, s);
    upload(bcg_bidx_, gi, s);
    bcg_cp_.alloc(3LL * static_cast<int64_t>(gchb.size()));
    bcg_sc_.alloc(5LL * nb_);
    bcg_fa_.alloc(nb_);
    bcg_fb_.alloc(nb_);
    bcg_done_.alloc(nb_);
    bcg_iters_.alloc(nb_);
    bcg_ndone_.alloc(1);
    dlam_prev_.alloc(nt_);
    body_have_prev_.alloc(1);
    MGPBD_CUDA(cudaMemsetAsync(body_have_prev_.p, 0, sizeof(int32_t), s));
    have_prev_ = false;
  }
  body_newton_d_.alloc(nb_);
  body_r0_d_.alloc(nb_);
  body_r_d_.alloc(nb_);
  body_bnorm_d_.alloc(nb_);
  body_sq_d_.alloc(nb_);
  body_cur_d_.alloc(nb_);
  body_omh_d_.alloc(nb_);
  body_loop_.alloc(1);
  body_log_.alloc(std::max(1, p_.maxiter) + 1);
  if (!h_body_loop_) MGPBD_CUDA(cudaMallocHost(&h_body_loop_, sizeof(BodyLoop)));
  drop_body_graph();
  MGPBD_CUDA(cudaStreamSynchronize(s));
}

void Solver::drop_body_graph() {
  if (body_exec_) {
    cudaGraphExecDestroy(body_exec_);
    body_exec_ = nullptr;
  }
}

BodyArrays Solver::body_arrays() {
  BodyArrays ba;
  ba.nb = nb_;
  ba.n_chunks = static_cast<int32_t>(chunk_body_.size());
  ba.chunk_ptr = body_chunk_ptr_.p;
  ba.chunk_idx = body_chunk_idx_.p;
  ba.partials = chunk_partials_.p;
  ba.active = body_active_.p;
  ba.r0 = body_r0_d_.p;
  ba.r = body_r_d_.p;
  ba.bnorm = body_bnorm_d_.p;
  ba.sq = body_sq_d_.p;
  ba.cur = body_cur_d_.p;
  ba.newton = body_newton_d_.p;
  ba.omega = body_omega_.p;
  ba.omega_h = body_omh_d_.p;
  ba.log = body_log_.p;
  ba.log_cap = static_cast<int32_t>(body_log_.n);
  return ba;
}

BodyLimits Solver::body_limits() const {
  BodyLimits lim;
  lim.atol = p_.atol;
  lim.rtol = p_.rtol;
  lim.tol_cg = p_.tol_cg;
  lim.rel_tol_cg = p_.rel_tol_cg;
  lim.maxiter = p_.maxiter;
  lim.maxiter_cg = p_.maxiter_cg;
  lim.per_body_cg = p_.body_cg ? 1 : 0;
  return lim;
}

BodyCg Solver::body_cg() {
  BodyCg b;
  b.nb = nb_;
  b.nch = static_cast<int32_t>(bcg_chb_.n);
  b.ch = reinterpret_cast<const int2*>(bcg_ch_.p);
  b.chb = bcg_chb_.p;
  b.bptr = bcg_bptr_.p;
  b.bidx = bcg_bidx_.p;
  b.cbody = cons_body_.p;
  b.cp = bcg_cp_.p;
  b.sc = bcg_sc_.p;
  b.fa = bcg_fa_.p;
  b.fb = bcg_fb_.p;
  b.done = bcg_done_.p;
  b.iters = bcg_iters_.p;
  b.ndone = bcg_ndone_.p;
  return b;
}

JcgVecs Solver::dual_vecs(const float* b, float* x) {
  JcgVecs v;
  v.b = b;
  v.x = x;
  v.xc = jxc_.p;
  v.r = jrf_.p;
  v.z = jz_.p;
  v.d = jd_.p;
  v.p = jp_.p;
  v.ap = jap_.p;
  v.partials = partials_.p;
  v.partials_capacity = static_cast<int64_t>(kMaxReduceBlocks) * 16;
  v.gs = jgs_.p;
  v.ulo = ulo_.p;
  return v;
}

// One CG per body (launch_jcg_bodies) to each body's own bound
// max(tol_cg, rel_tol_cg |b_b|).
int32_t Solver::run_dual_bodies(const float* b, float* x, int32_t maxit, bool warm) {
  cudaStream_t outer = stream_;
  const JcgVecs v = dual_vecs(b, x);
  MGPBD_CUDA(cudaEventRecord(ev_[0], outer));
  dual_x_ = nullptr;
  launch_jcg_bodies(jview(), v, body_cg(), jst_.p, cg_state_.p, p_.tol_cg, p_.rel_tol_cg, maxit,
                    p_.cheb_degree, warm, barrier_limit_s_, outer);
  dual_x_ = x;
  MGPBD_CUDA(cudaEventRecord(ev_[1], outer));
  sync_read(h_state_, cg_state_.p, sizeof(CgState));
  stats_.ms_dual += event_ms(ev_[0], ev_[1]);
  stats_.cg_launches += 1;
  if (static_cast<uint32_t>(h_state_->status) & MGPBD_STATUS_SYNC_TIMEOUT) {
    status_ |= MGPBD_STATUS_SYNC_TIMEOUT;
    throw Error(MGPBD_ECUDA, "persistent CG kernel: a grid barrier wait timed out");
  }
  status_ |= static_cast<uint32_t>(h_state_->status);
  return h_state_->iters;
}

// out[k * nb + b] = sum of the chunk partials k of body b, in chunk order
void Solver::chunk_body_sums(int count, std::vector<double>& out) {
  const int64_t nc = static_cast<int64_t>(chunk_body_.size());
  std::vector<double> h(count * nc);
  MGPBD_CUDA(cudaMemcpyAsync(h.data(), chunk_partials_.p, sizeof(double) * h.size(),
                             cudaMemcpyDeviceToHost, stream_));
  MGPBD_CUDA(cudaStreamSynchronize(stream_));
  out.assign(static_cast<size_t>(count) * nb_, 0.0);
  for (int k = 0; k < count; ++k)
    for (int64_t c = 0; c < nc; ++c) out[static_cast<size_t>(k) * nb_ + chunk_body_[c]] += h[k * nc + c];
}

// The block-diagonal CG solve of one Newton iteration, verified per body:
// CG to |r| <= rel |b| over the batch, then each body's own residual
// |r_b| <= rel |b_b| is checked; while some body misses it, CG continues
// from its iterate (float64 restart residual) to the smallest missing
// body's bound.  bnorm[b] = |b_b| (0 for bodies whose loop has ended).
int32_t Solver::pcg_bodies(const float* b, float* x, const std::vector<double>& bnorm) {
  if (p_.body_cg) {
    const bool warm = warm_next_;
    warm_next_ = false;
    return run_dual_bodies(b, x, p_.maxiter_cg, warm);
  }
  const double rel = p_.rel_tol_cg;
  const int32_t n_ch = static_cast<int32_t>(chunk_body_.size());
  double bn2 = 0.0;
  for (double v : bnorm) bn2 += v * v;
  double tol = std::max<double>(p_.tol_cg, rel * std::sqrt(bn2));
  int32_t total = 0, left = p_.maxiter_cg;
  bool warm = false;
  std::vector<double> rb2;
  for (int pass = 0; pass < 6 && left > 0; ++pass) {
    const int32_t its = run_dual(b, x, tol, 0.0, left, warm, ulo_.p);
    total += its;
    left -= its;
    if (status_ & (MGPBD_STATUS_NAN | MGPBD_STATUS_PAP_NONPOS)) break;
    launch_chunk_dual_sq(jrf_.p, nullptr, nullptr, chunks_.p, n_ch, chunk_partials_.p, stream_);
    chunk_body_sums(1, rb2);
    double need = std::numeric_limits<double>::infinity();
    for (int32_t k = 0; k < nb_; ++k) {
      const double bound = std::max<double>(p_.tol_cg, rel * bnorm[k]);
      if (bnorm[k] > 0.0 && std::sqrt(rb2[k]) > bound) need = std::min(need, bound);
    }
    if (!std::isfinite(need)) return total;
    tol = need;
    warm = true;
  }
  status_ |= MGPBD_STATUS_CG_MAXITER;
  return total;
}

// The Newton loop of cons/mgpbd_gpu.py:397-446 run per body: each body's
// residual, stopping test and line-search step are its own; bodies whose
// test holds keep their positions (zero right-hand side) while the others
// go on.
void Solver::solve_bodies() {
  cudaStream_t s = stream_;
  status_ = 0;
  MGPBD_CUDA(cudaMemsetAsync(lambda_.p, 0, sizeof(float) * nt_, s));
  stats_.newton_iters = 0;
  stats_.cg_iters_total = 0;
  stats_.cg_iters_last = 0;
  stats_.omega_last = 1.0;
  stats_.cg_iters_warm = 0;
  stats_.cg_launches = 0;
  stats_.ms_warm = 0.0;
  stats_.ms_dual = 0.0;
  stats_.warm_amp = 0.0;
  stats_.warm_declined = 0;
  log_.clear();
  auto now = [] {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  };
  const int32_t n_ch = static_cast<int32_t>(chunk_body_.size());
  std::vector<int32_t> active(nb_, 1);
  std::vector<double> r2, bnorm(nb_), cur, trial;
  std::vector<float> om(nb_);
  std::fill(body_newton_.begin(), body_newton_.end(), 0);
  std::fill(body_omega_h_.begin(), body_omega_h_.end(), 1.0);
  for (int32_t ite = 0; ite < p_.maxiter; ++ite) {
    compute_constraints();
    launch_rhs(C_.p, alpha_.p, lambda_.p, nt_, rhs_.p, partials_.p, s);
    launch_chunk_dual_sq(C_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, s);
    chunk_body_sums(1, r2);
    double rg2 = 0.0;
    for (double v : r2) rg2 += v;
    const double r = std::sqrt(rg2);
    if (ite == 0) {
      stats_.residual0 = r;
      for (int32_t k = 0; k < nb_; ++k) body_r0_[k] = std::sqrt(r2[k]);
    }
    stats_.residual = r;
    if (!std::isfinite(r)) {
      status_ |= MGPBD_STATUS_NAN;
      break;
    }
    int32_t n_active = 0;
    for (int32_t k = 0; k < nb_; ++k) {
      bnorm[k] = 0.0;
      if (!active[k]) continue;
      const double rk = std::sqrt(r2[k]);
      body_r_[k] = rk;
      if (rk < p_.atol || (body_r0_[k] > 1e-12 && rk < p_.rtol * body_r0_[k])) {
        active[k] = 0;
      } else {
        bnorm[k] = rk;
        ++n_active;
      }
    }
    if (n_active == 0) {
      log_.push_back({double(ite), r, 0.0, 1.0, now()});
      break;
    }
    MGPBD_CUDA(cudaMemcpyAsync(body_active_.p, active.data(), sizeof(int32_t) * nb_,
                               cudaMemcpyHostToDevice, s));
    launch_mask_rhs(rhs_.p, cons_body_.p, body_active_.p, nt_, s);
    fill_matrices();
    dual_x_ = nullptr;
    const bool warm_sub = ite == 0 && p_.warm_substep && p_.body_cg;
    if (warm_sub && have_prev_) {
      MGPBD_CUDA(cudaMemcpyAsync(dlam_.p, dlam_prev_.p, sizeof(float) * nt_,
                                 cudaMemcpyDeviceToDevice, s));
      warm_next_ = true;
    }
    const int32_t it = pcg_bodies(rhs_.p, dlam_.p, bnorm);
    warm_next_ = false;
    if (warm_sub && !(status_ & (MGPBD_STATUS_NAN | MGPBD_STATUS_CG_MAXITER))) {
      MGPBD_CUDA(cudaMemcpyAsync(dlam_prev_.p, dlam_.p, sizeof(float) * nt_,
                                 cudaMemcpyDeviceToDevice, s));
      have_prev_ = true;
    }
    scatter(dlam_.p);
    // per-body line search (cons/mgpbd_gpu.py:379-391): the first of 1,
    // 1/2, ..., 1/512 whose dual norm (updated lambda) beats the current one
    launch_chunk_dual_sq(C_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, s);
    chunk_body_sums(1, cur);
    double steps[kBodyTrials];
    for (int k = 0; k < kBodyTrials; ++k) steps[k] = std::ldexp(1.0, -k);
    std::memcpy(h_buf_, steps, sizeof(steps));
    MGPBD_CUDA(cudaMemcpyAsync(omegas_.p, h_buf_, sizeof(steps), cudaMemcpyHostToDevice, s));
    launch_chunk_trial(x_, dpos_.p, omegas_.p, 1, t_i_, ctype_.p, dm_inv_.p, rest_vol_.p,
                       alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, s);
    chunk_body_sums(1, trial);
    bool more = false;
    for (int32_t k = 0; k < nb_; ++k) {
      om[k] = 1.0f;
      if (active[k] && !(std::sqrt(trial[k]) < std::sqrt(cur[k]))) more = true;
    }
    if (more) {
      launch_chunk_trial(x_, dpos_.p, omegas_.p, kBodyTrials, t_i_, ctype_.p, dm_inv_.p,
                         rest_vol_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, s);
      chunk_body_sums(kBodyTrials, trial);
      for (int32_t k = 0; k < nb_; ++k) {
        if (!active[k]) continue;
        double w = std::ldexp(1.0, -kBodyTrials);
        for (int q = 0; q < kBodyTrials; ++q)
          if (std::sqrt(trial[static_cast<size_t>(q) * nb_ + k]) < std::sqrt(cur[k])) {
            w = steps[q];
            break;
          }
        om[k] = static_cast<float>(w);
      }
    }
    MGPBD_CUDA(cudaMemcpyAsync(body_omega_.p, om.data(), sizeof(float) * nb_,
                               cudaMemcpyHostToDevice, s));
    launch_apply_bodies(x_, dpos_.p, invm_, vert_body_.p, body_omega_.p, nv_, s);
    double om_min = 1.0;
    for (int32_t k = 0; k < nb_; ++k)
      if (active[k]) {
        body_newton_[k] += 1;
        body_omega_h_[k] = om[k];
        om_min = std::min<double>(om_min, om[k]);
      }
    log_.push_back({double(ite), r, double(it), om_min, now()});
    stats_.newton_iters = ite + 1;
    stats_.cg_iters_total += it;
    stats_.cg_iters_last = it;
    stats_.omega_last = om_min;
    if (ite + 1 == p_.maxiter) status_ |= MGPBD_STATUS_NEWTON_MAXITER;
  }
  stats_.status = status_;
}

// The Newton loop of solve_bodies as one CUDA graph: the residual and
// stopping tests before the loop, then a device-side while loop whose body
// is one Newton iteration: masked right-hand side, Lanczos estimate and
// Chebyshev coefficients, up to 6 verified CG passes (the persistent
// kernel with its tolerance, limit and start read from the device; unused
// passes return at once), scatter, the per-body line search over all 10
// steps, the position update, and the next residual, which decides whether
// the loop goes on.  Decisions are the host loop's (bodies.cu).
void Solver::capture_body_graph() {
  drop_body_graph();
  cudaStream_t outer = stream_;
  cudaStream_t cs, bs;
  MGPBD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  MGPBD_CUDA(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  const int32_t n_ch = static_cast<int32_t>(chunk_body_.size());
  const BodyArrays ba = body_arrays();
  const BodyLimits lim = body_limits();
  BodyLoop* L = body_loop_.p;
  const JcgVecs v = dual_vecs(rhs_.p, dlam_.p);
  try {
    long long c0 = g_launches.load();
    MGPBD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    stream_ = cs;
    MGPBD_CUDA(cudaMemsetAsync(lambda_.p, 0, sizeof(float) * nt_, cs));
    launch_bodies_reset(ba, L, cs);
    compute_constraints();
    launch_rhs(C_.p, alpha_.p, lambda_.p, nt_, rhs_.p, partials_.p, cs);
    launch_chunk_dual_sq(C_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, cs);
    cudaStreamCaptureStatus cst;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    MGPBD_CUDA(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &graph, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle handle;
    MGPBD_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault));
    launch_bodies_residual(ba, L, lim, handle, cs);
    MGPBD_CUDA(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &graph, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond;
    MGPBD_CUDA(cudaGraphAddNode(&cond, graph, deps, nullptr, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    MGPBD_CUDA(cudaStreamUpdateCaptureDependencies(cs, &cond, nullptr, 1, cudaStreamSetCaptureDependencies));
    long long c1 = g_launches.load();
    MGPBD_CUDA(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    stream_ = bs;
    launch_mask_rhs(rhs_.p, cons_body_.p, body_active_.p, nt_, bs);
    jform_setup(&L->status);
    if (p_.body_cg) {
      if (p_.warm_substep)
        launch_bodies_warm_in(L, body_have_prev_.p, dlam_.p, dlam_prev_.p, nt_, bs);
      launch_jcg_bodies(jview(), v, body_cg(), jst_.p, cg_state_.p, p_.tol_cg, p_.rel_tol_cg,
                        p_.maxiter_cg, p_.cheb_degree, false, barrier_limit_s_, bs, &L->jc);
      launch_bodies_verify(ba, L, cg_state_.p, lim, bs);
      if (p_.warm_substep)
        launch_bodies_warm_out(L, body_have_prev_.p, dlam_.p, dlam_prev_.p, nt_, bs);
    } else {
      for (int pass = 0; pass < 6; ++pass) {
        launch_jcg_persistent(jview(), v, jplan_, jpart_.p, jst_.p, cg_state_.p, p_.tol_cg, 0.0,
                              p_.maxiter_cg, p_.cheb_degree, false, barrier_limit_s_, bs, &L->jc);
        launch_chunk_dual_sq(jrf_.p, nullptr, nullptr, chunks_.p, n_ch, chunk_partials_.p, bs);
        launch_bodies_verify(ba, L, cg_state_.p, lim, bs);
      }
    }
    dual_x_ = dlam_.p;
    scatter(dlam_.p);
    launch_chunk_dual_sq(C_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, bs);
    launch_bodies_cur(ba, bs);
    launch_chunk_trial(x_, dpos_.p, omegas_.p, kBodyTrials, t_i_, ctype_.p, dm_inv_.p,
                       rest_vol_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, bs);
    launch_bodies_omega(ba, L, lim, kBodyTrials, bs);
    launch_apply_bodies(x_, dpos_.p, invm_, vert_body_.p, body_omega_.p, nv_, bs);
    compute_constraints();
    launch_rhs(C_.p, alpha_.p, lambda_.p, nt_, rhs_.p, partials_.p, bs);
    launch_chunk_dual_sq(C_.p, alpha_.p, lambda_.p, chunks_.p, n_ch, chunk_partials_.p, bs);
    launch_bodies_residual(ba, L, lim, handle, bs);
    long long c2 = g_launches.load();
    MGPBD_CUDA(cudaStreamEndCapture(bs, &body));
    stream_ = outer;
    MGPBD_CUDA(cudaStreamEndCapture(cs, &graph));
    g_launches.fetch_sub(c2 - c0);
    body_graph_init_launches_ = c1 - c0;
    body_graph_body_launches_ = c2 - c1;
    MGPBD_CUDA(cudaGraphInstantiate(&body_exec_, graph, 0));
    cudaGraphDestroy(graph);
  } catch (...) {
    stream_ = outer;
    cudaStreamCaptureStatus cst;
    if (cudaStreamIsCapturing(bs, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
      cudaGraph_t g2;
      cudaStreamEndCapture(bs, &g2);
    }
    if (cudaStreamIsCapturing(cs, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
      cudaGraph_t g2 = nullptr;
      cudaStreamEndCapture(cs, &g2);
      if (g2) cudaGraphDestroy(g2);
    }
    cudaGetLastError();
    cudaStreamDestroy(cs);
    cudaStreamDestroy(bs);
    throw;
  }
  cudaStreamDestroy(cs);
  cudaStreamDestroy(bs);
  body_exec_limit_ = barrier_limit_s_;
}

void Solver::solve_bodies_graph() {
  cudaStream_t s = stream_;
  require(p_.maxiter + 1 <= static_cast<int32_t>(body_log_.n), MGPBD_ESTATE,
          "bodies: the loop log is smaller than maxiter + 1");
  if (!body_exec_ || body_exec_limit_ != barrier_limit_s_) capture_body_graph();
  // the line-search steps 1, 1/2, ..., 1/512 (the graph reads them)
  double steps[kBodyTrials];
  for (int k = 0; k < kBodyTrials; ++k) steps[k] = std::ldexp(1.0, -k);
  std::memcpy(h_buf_, steps, sizeof(steps));
  MGPBD_CUDA(cudaMemcpyAsync(omegas_.p, h_buf_, sizeof(steps), cudaMemcpyHostToDevice, s));
  MGPBD_CUDA(cudaEventRecord(ev_[0], s));
  MGPBD_CUDA(cudaGraphLaunch(body_exec_, s));
  MGPBD_CUDA(cudaEventRecord(ev_[1], s));
  MGPBD_CUDA(cudaMemcpyAsync(h_body_loop_, body_loop_.p, sizeof(BodyLoop), cudaMemcpyDeviceToHost, s));
  std::vector<BodyLogEntry> lg(body_log_.n);
  MGPBD_CUDA(cudaMemcpyAsync(lg.data(), body_log_.p, sizeof(BodyLogEntry) * lg.size(),
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaMemcpyAsync(body_newton_.data(), body_newton_d_.p, sizeof(int32_t) * nb_,
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaMemcpyAsync(body_r0_.data(), body_r0_d_.p, sizeof(double) * nb_,
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaMemcpyAsync(body_r_.data(), body_r_d_.p, sizeof(double) * nb_,
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaMemcpyAsync(body_omega_h_.data(), body_omh_d_.p, sizeof(double) * nb_,
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
  const BodyLoop& L = *h_body_loop_;
  g_launches.fetch_add(body_graph_init_launches_ + body_graph_body_launches_ * L.ite);
  status_ = L.status;
  stats_.newton_iters = L.ite;
  stats_.cg_iters_total = L.cg_total;
  stats_.cg_iters_last = L.ite > 0 ? static_cast<int32_t>(lg[L.ite - 1].cg) : 0;
  stats_.omega_last = L.omega_min;
  stats_.residual0 = L.residual0;
  stats_.residual = L.residual;
  stats_.cg_iters_warm = 0;
  stats_.cg_launches = L.cg_launches;
  stats_.ms_warm = 0.0;
  stats_.ms_dual = event_ms(ev_[0], ev_[1]);
  stats_.warm_amp = 0.0;
  stats_.warm_declined = 0;
  stats_.status = status_;
  log_.clear();
  const double t = std::chrono::duration<double>(
                       std::chrono::steady_clock::now().time_since_epoch()).count();
  for (int32_t i = 0; i < L.n_log && i < static_cast<int32_t>(lg.size()); ++i)
    log_.push_back({double(i), lg[i].r, lg[i].cg, lg[i].omega, t});
  if (status_ & MGPBD_STATUS_SYNC_TIMEOUT)
    throw Error(MGPBD_ECUDA, "persistent CG kernel: a grid barrier wait timed out");
}

void Solver::body_stats(int32_t n, int32_t* newton, double* r0, double* r, double* omega) const {
  require(n == nb_ && nb_ > 0, MGPBD_EINVAL, "body_stats: n must equal the number of bodies");
  for (int32_t k = 0; k < nb_; ++k) {
    if (newton) newton[k] = body_newton_[k];
    if (r0) r0[k] = body_r0_[k];
    if (r) r[k] = body_r_[k];
    if (omega) omega[k] = body_omega_h_[k];
  }
}

void* Solver::field(int32_t id, int64_t* count) {
  require_init();
  switch (id) {
    case MGPBD_FIELD_LAMBDA: *count = nt_; return lambda_.p;
    case MGPBD_FIELD_CONSTRAINTS: *count = nt_; return C_.p;
    case MGPBD_FIELD_GRADC: *count = 12LL * nt_; return gradC_.p;
    case MGPBD_FIELD_ALPHA_TILDE: *count = nt_; return alpha_.p;
    case MGPBD_FIELD_REST_VOL: *count = nt_; return rest_vol_.p;
    case MGPBD_FIELD_DM_INV: *count = 9LL * nt_; return dm_inv_.p;
    case MGPBD_FIELD_X_OLD: *count = 3LL * nv_; return x_old_.p;
    case MGPBD_FIELD_X_PREDICT: *count = 3LL * nv_; return x_pred_.p;
    case MGPBD_FIELD_DPOS: *count = 3LL * nv_; return dpos_.p;
    case MGPBD_FIELD_RHS: *count = nt_; return rhs_.p;
    case MGPBD_FIELD_DLAMBDA: *count = nt_; return dlam_.p;
    case MGPBD_FIELD_A_DATA: *count = levels_[0].nnz; return levels_[0].data.p;
    default: throw Error(MGPBD_EINVAL, "unknown field id");
  }
}

const Level& Solver::level(int32_t l) const {
  require_init();
  require(l >= 0 && l < n_levels(), MGPBD_EINVAL, "level out of range");
  return levels_[l];
}

}  // namespace mgpbd
