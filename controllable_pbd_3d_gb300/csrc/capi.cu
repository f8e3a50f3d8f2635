// extern "C" entry points of libmgpbd.so (declared in include/mgpbd.h).
// Every call catches C++ exceptions and returns an MGPBD_E* code; the text
// of the last error of the calling thread is available from
// mgpbd_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "common.h"
#include "../../include/mgpbd_local.h"
#include "coloring.h"
#include "kernels.cuh"
#include "local.cuh"
#include "mpnn.cuh"
#include "rap.cuh"
#include "solver.h"
#include "structure.h"

struct mgpbd_solver {
  mgpbd::Solver impl;
  explicit mgpbd_solver(const mgpbd_params& p) : impl(p) {}
};
struct mgpbd_net {
  mgpbd::CoarseNet impl;
  explicit mgpbd_net(uint64_t seed) : impl(seed) {}
};
struct mgpbd_xpbd {
  mgpbd::Xpbd impl;
  explicit mgpbd_xpbd(const mgpbd_xpbd_params& p) : impl(p) {}
};
struct mgpbd_vbd {
  mgpbd::Vbd impl;
  explicit mgpbd_vbd(const mgpbd_vbd_params& p) : impl(p) {}
};

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F&& f) {
  try {
    f();
    return MGPBD_OK;
  } catch (const mgpbd::Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return MGPBD_ENOMEM;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return MGPBD_EINVAL;
  } catch (const std::length_error& e) {
    g_last_error = e.what();
    return MGPBD_ERANGE;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return MGPBD_EINVAL;
  }
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace

void mgpbd::set_last_error(const std::string& msg) { g_last_error = msg; }

namespace {

// copies a colouring into caller arrays of the documented capacities
void put_coloring(const mgpbd::Coloring& c, int32_t* ordered, int32_t* offsets, int32_t* n_colors) {
  std::copy(c.ordered.begin(), c.ordered.end(), ordered);
  std::copy(c.offsets.begin(), c.offsets.end(), offsets);
  *n_colors = c.n_colors;
}

}  // namespace

extern "C" {

void mgpbd_default_params(mgpbd_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->dt = 0.0f;
  p->mu = 1e6f;
  p->damp = 1.0f;
  p->maxiter = 20;
  p->atol = 1e-4f;
  p->rtol = 1e-2f;
  p->maxiter_cg = 100;
  p->tol_cg = 1e-5f;
  p->n_smooth = 2;
  p->omega_jacobi = 2.0f / 3.0f;
  p->setup_interval = 10000;
  p->use_line_search = 1;
  p->mode = MGPBD_MODE_PARITY;
  p->rel_tol_cg = 0.0f;
  p->coarse_solver = MGPBD_COARSE_JACOBI;
  p->smoother = MGPBD_SMOOTH_JACOBI;
  p->max_levels = 0;
  p->max_coarse = 400;
  p->kinematic_pins = 0;
  p->coarse_sweeps = 0;
  p->cg_alias = 0;
  p->compliance = 0.0f;
  p->precond = MGPBD_PRECOND_VCYCLE;
  p->cheb_degree = 8;
  p->cheb_lo = 0.01f;
  p->use_graph = 1;
  p->persistent = 1;
  p->primal = 0;
  p->primal_tol = 1e-2f;
  p->learned_accept = 0.1f;
  p->learned_stall = 1000;
  p->cheb_scale = MGPBD_CHEB_JACOBI;
  p->body_cg = 1;
  p->warm_substep = 0;
}

const char* mgpbd_strerror(int code) {
  switch (code) {
    case MGPBD_OK: return "ok";
    case MGPBD_EINVAL: return "invalid argument";
    case MGPBD_ECUDA: return "CUDA runtime error";
    case MGPBD_ENOMEM: return "out of memory";
    case MGPBD_ESTATE: return "call out of order";
    case MGPBD_ENUMERIC: return "non-finite value in the solve";
    case MGPBD_ERANGE: return "size out of range";
    case MGPBD_ENOTSUP: return "not supported";
    default: return "unknown error";
  }
}

const char* mgpbd_last_error(void) { return g_last_error.c_str(); }

const char* mgpbd_version(void) { return "mgpbd-gb300 0.1 (sm_103a)"; }

int64_t mgpbd_launch_count(void) { return mgpbd::g_launches.load(); }

int mgpbd_create(const mgpbd_params* params, mgpbd_handle* out) {
  if (!params || !out) return MGPBD_EINVAL;
  *out = nullptr;
  return guarded([&] { *out = new mgpbd_solver(*params); });
}

void mgpbd_destroy(mgpbd_handle h) { delete h; }

int mgpbd_set_stream(mgpbd_handle h, void* stream) {
  if (!h) return MGPBD_EINVAL;
  h->impl.set_stream(as_stream(stream));
  return MGPBD_OK;
}

int mgpbd_set_mesh(mgpbd_handle h, const float* x_ref, const float* invm, const int32_t* t_i,
                   int32_t nv, int32_t nt, float* x, float* v) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_mesh(x_ref, invm, t_i, nv, nt, x, v); });
}

int mgpbd_set_hierarchy(mgpbd_handle h, const int32_t* agg_ids, int32_t n_levels,
                        const int32_t* level_sizes) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_hierarchy(agg_ids, n_levels, level_sizes); });
}

int mgpbd_set_matrix(mgpbd_handle h, int32_t n, int64_t nnz, const int32_t* indptr,
                     const int32_t* indices, const float* data) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_matrix(n, nnz, indptr, indices, data); });
}

int mgpbd_update_matrix(mgpbd_handle h, const float* data) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.update_matrix(data); });
}

int mgpbd_set_bodies(mgpbd_handle h, int32_t n_bodies, const int32_t* vert_off, int32_t n_segs,
                     const int32_t* segs) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_bodies(n_bodies, vert_off, n_segs, segs); });
}

int mgpbd_body_stats(mgpbd_handle h, int32_t n, int32_t* newton_iters, double* residual0,
                     double* residual, double* omega) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.body_stats(n, newton_iters, residual0, residual, omega); });
}

int mgpbd_set_barrier_limit(mgpbd_handle h, double seconds) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_barrier_limit(seconds); });
}

int mgpbd_init(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.init(); });
}

int mgpbd_step(mgpbd_handle h, int32_t frame) {
  if (!h) return MGPBD_EINVAL;
  int rc = guarded([&] { h->impl.step(frame); });
  if (rc == MGPBD_OK && (h->impl.status() & MGPBD_STATUS_NAN)) return MGPBD_ENUMERIC;
  return rc;
}

int mgpbd_make_prediction(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.make_prediction(); });
}

int mgpbd_solve(mgpbd_handle h, int32_t frame) {
  if (!h) return MGPBD_EINVAL;
  int rc = guarded([&] { h->impl.solve(frame); });
  if (rc == MGPBD_OK && (h->impl.status() & MGPBD_STATUS_NAN)) return MGPBD_ENUMERIC;
  return rc;
}

int mgpbd_update_vel(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.update_vel(); });
}

int mgpbd_get_stats(mgpbd_handle h, mgpbd_stats* out) {
  if (!h || !out) return MGPBD_EINVAL;
  *out = h->impl.stats();
  return MGPBD_OK;
}

int mgpbd_newton_log(mgpbd_handle h, int32_t max_rows, double* rows, int32_t* n_rows) {
  if (!h || !n_rows || max_rows < 0 || (max_rows > 0 && !rows)) return MGPBD_EINVAL;
  const auto& log = h->impl.newton_log();
  *n_rows = static_cast<int32_t>(log.size());
  int32_t m = std::min<int32_t>(max_rows, *n_rows);
  for (int32_t i = 0; i < m; ++i)
    for (int k = 0; k < 5; ++k) rows[5 * i + k] = log[i][k];
  return MGPBD_OK;
}

int mgpbd_get_status(mgpbd_handle h, uint32_t* status) {
  if (!h || !status) return MGPBD_EINVAL;
  *status = h->impl.status();
  return MGPBD_OK;
}

int mgpbd_field(mgpbd_handle h, int32_t field, void** dev_ptr, int64_t* count) {
  if (!h || !dev_ptr || !count) return MGPBD_EINVAL;
  return guarded([&] { *dev_ptr = h->impl.field(field, count); });
}

int mgpbd_level_csr(mgpbd_handle h, int32_t level, int32_t* n_rows, int64_t* nnz, int32_t** indptr,
                    int32_t** indices, float** data, float** diag_inv) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] {
    const mgpbd::Level& L = h->impl.level(level);
    if (n_rows) *n_rows = L.n;
    if (nnz) *nnz = L.nnz;
    if (indptr) *indptr = L.indptr.p;
    if (indices) *indices = L.indices.p;
    if (data) *data = L.data.p;
    if (diag_inv) *diag_inv = L.diag_inv.p;
  });
}

int mgpbd_level_agg(mgpbd_handle h, int32_t level, int32_t** agg_ids) {
  if (!h || !agg_ids) return MGPBD_EINVAL;
  return guarded([&] {
    const mgpbd::Level& L = h->impl.level(level);
    mgpbd::require(L.agg.p != nullptr, MGPBD_EINVAL, "level has no coarser level");
    *agg_ids = L.agg.p;
  });
}

int mgpbd_level_count(mgpbd_handle h, int32_t* n_levels) {
  if (!h || !n_levels) return MGPBD_EINVAL;
  return guarded([&] { *n_levels = h->impl.n_levels(); });
}

int mgpbd_compute_constraints(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.compute_constraints(); });
}

int mgpbd_fill_matrices(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.fill_matrices(); });
}

int mgpbd_refill_coarse(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.refill_coarse(); });
}

int mgpbd_compute_rhs(mgpbd_handle h, double* residual_norm) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] {
    double r = h->impl.compute_rhs();
    if (residual_norm) *residual_norm = r;
  });
}

int mgpbd_pcg(mgpbd_handle h, const float* b, float* x, int32_t* cg_iters) {
  if (!h || !b || !x) return MGPBD_EINVAL;
  return guarded([&] {
    int32_t it = h->impl.pcg(b, x);
    if (cg_iters) *cg_iters = it;
  });
}

// ---- learned coarse correction -------------------------------------------

namespace {
mgpbd::NetGraph net_graph(int32_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                          const float* data, const float* diag_inv) {
  mgpbd::require(n > 0 && nnz >= n && indptr && indices && data && diag_inv, MGPBD_EINVAL,
                 "net: empty graph, nnz < n or null CSR array");
  mgpbd::NetGraph g;
  g.n = n;
  g.nnz = nnz;
  g.indptr = indptr;
  g.indices = indices;
  g.data = data;
  g.diag_inv = diag_inv;
  return g;
}
}  // namespace

int mgpbd_net_create(uint64_t seed, mgpbd_net_handle* out) {
  if (!out) return MGPBD_EINVAL;
  *out = nullptr;
  return guarded([&] { *out = new mgpbd_net(seed); });
}

void mgpbd_net_destroy(mgpbd_net_handle net) { delete net; }

int mgpbd_net_params(mgpbd_net_handle net, float** params, float** grad) {
  if (!net) return MGPBD_EINVAL;
  if (params) *params = net->impl.params();
  if (grad) *grad = net->impl.grad();
  return MGPBD_OK;
}

int mgpbd_net_sync_params(mgpbd_net_handle net, void* stream) {
  if (!net) return MGPBD_EINVAL;
  return guarded([&] { net->impl.sync_params(as_stream(stream)); });
}

int mgpbd_net_forward(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                      const int32_t* indices, const float* data, const float* diag_inv,
                      const float* r, float* e, void* stream) {
  if (!net || !r || !e) return MGPBD_EINVAL;
  return guarded([&] {
    net->impl.forward(net_graph(n, nnz, indptr, indices, data, diag_inv), r, e, as_stream(stream));
  });
}

int mgpbd_net_weights(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                      const int32_t* indices, const float* data, const float* diag_inv,
                      float* w, void* stream) {
  if (!net || !w) return MGPBD_EINVAL;
  return guarded([&] {
    net->impl.weights(net_graph(n, nnz, indptr, indices, data, diag_inv), w, as_stream(stream));
  });
}

int mgpbd_net_apply(int32_t n, const float* w, const float* diag_inv, const float* r, float* e,
                    void* stream) {
  if (n < 0 || (n > 0 && (!w || !diag_inv || !r || !e))) return MGPBD_EINVAL;
  return guarded([&] {
    if (n > 0) mgpbd::apply_coarse_weights(n, w, diag_inv, r, e, as_stream(stream));
  });
}

int mgpbd_net_loss_grad(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                        const int32_t* indices, const float* data, const float* diag_inv,
                        const float* samples, int32_t n_samples, int32_t mode, double* loss,
                        void* stream) {
  if (!net || !samples || n_samples <= 0) return MGPBD_EINVAL;
  return guarded([&] {
    cudaStream_t s = as_stream(stream);
    mgpbd::DevBuf<double> d(1);
    net->impl.loss_grad(net_graph(n, nnz, indptr, indices, data, diag_inv), samples, n_samples, 0,
                        n_samples, d.p, mode, s);
    double h = 0.0;
    MGPBD_CUDA(cudaMemcpyAsync(&h, d.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    MGPBD_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = h;
  });
}

int mgpbd_net_adam(mgpbd_net_handle net, float lr, float beta1, float beta2, float eps,
                   void* stream) {
  if (!net) return MGPBD_EINVAL;
  return guarded([&] { net->impl.adam(lr, beta1, beta2, eps, as_stream(stream)); });
}

int mgpbd_net_train(mgpbd_net_handle net, int32_t n, int64_t nnz, const int32_t* indptr,
                    const int32_t* indices, const float* data, const float* diag_inv,
                    const float* samples, int32_t n_samples, int32_t batch, int32_t steps,
                    float lr, double* losses, void* stream) {
  if (!net || !samples || n_samples <= 0 || batch <= 0 || steps < 0) return MGPBD_EINVAL;
  return guarded([&] {
    if (steps == 0) return;
    cudaStream_t s = as_stream(stream);
    mgpbd::DevBuf<double> d(steps);
    net->impl.train(net_graph(n, nnz, indptr, indices, data, diag_inv), samples, n_samples, batch,
                    steps, lr, d.p, s);
    std::vector<double> h(steps);
    MGPBD_CUDA(cudaMemcpyAsync(h.data(), d.p, sizeof(double) * steps, cudaMemcpyDeviceToHost, s));
    MGPBD_CUDA(cudaStreamSynchronize(s));
    if (losses) std::copy(h.begin(), h.end(), losses);
  });
}

int mgpbd_autotune_rows(mgpbd_handle h, int32_t reps, int32_t* codes, float* us_per_sweep) {
  if (!h || reps < 1) return MGPBD_EINVAL;
  return guarded([&] { h->impl.autotune_rows(reps, codes, us_per_sweep); });
}

int mgpbd_level_row_shape(mgpbd_handle h, int32_t level, int32_t* code) {
  if (!h || !code) return MGPBD_EINVAL;
  return guarded([&] { *code = h->impl.level_row_shape(level); });
}

int mgpbd_set_level_row_shape(mgpbd_handle h, int32_t level, int32_t code) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_level_row_shape(level, code); });
}

int mgpbd_row_shapes(int32_t* codes, int32_t* count) {
  if (!count) return MGPBD_EINVAL;
  return guarded([&] {
    if (codes)
      for (int i = 0; i < mgpbd::kNumRowShapes; ++i) codes[i] = mgpbd::row_shape_code(i);
    *count = mgpbd::kNumRowShapes;
  });
}

int mgpbd_set_constraint_types(mgpbd_handle h, const int32_t* types) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_constraint_types(types); });
}

int mgpbd_set_coarse_net(mgpbd_handle h, mgpbd_net_handle net) {
  if (!h) return MGPBD_EINVAL;
  h->impl.set_coarse_net(net ? &net->impl : nullptr);
  return MGPBD_OK;
}

int mgpbd_record_coarse(mgpbd_handle h, float* rc, float* ec, int32_t capacity, int32_t every) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.record_coarse(rc, ec, capacity, every); });
}

int mgpbd_record_count(mgpbd_handle h, int32_t* count) {
  if (!h || !count) return MGPBD_EINVAL;
  *count = h->impl.record_count();
  return MGPBD_OK;
}

int mgpbd_vcycle(mgpbd_handle h, const float* r, float* z) {
  if (!h || !r || !z) return MGPBD_EINVAL;
  return guarded([&] { h->impl.vcycle_into(r, z); });
}

int mgpbd_scatter(mgpbd_handle h, const float* dlam) {
  if (!h || !dlam) return MGPBD_EINVAL;
  return guarded([&] { h->impl.scatter(dlam); });
}

int mgpbd_line_search(mgpbd_handle h, double* omega) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] {
    double w = h->impl.line_search();
    if (omega) *omega = w;
  });
}

int mgpbd_apply_dpos(mgpbd_handle h, double omega) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.apply_dpos(omega); });
}

int mgpbd_apply_matrix(mgpbd_handle h, int32_t matrix_free, const float* x, float* y) {
  if (!h || !x || !y) return MGPBD_EINVAL;
  if (matrix_free < 0 || matrix_free > 2) return MGPBD_EINVAL;
  return guarded([&] { h->impl.apply_matrix(matrix_free, x, y); });
}

int mgpbd_zone_proximity(mgpbd_handle h, int32_t* active, float cx, float cy, float cz,
                         float radius) {
  if (!h || !active) return MGPBD_EINVAL;
  return guarded([&] { h->impl.zone_proximity(active, cx, cy, cz, radius); });
}

int mgpbd_zone_strain(mgpbd_handle h, int32_t* active, const float* x_old, float threshold,
                      float dt) {
  if (!h || !active || !(dt > 0.0f)) return MGPBD_EINVAL;
  return guarded([&] { h->impl.zone_strain(active, x_old, threshold, dt); });
}

int mgpbd_zone_expand(mgpbd_handle h, int32_t* active, int32_t n_rings) {
  if (!h || !active || n_rings < 0) return MGPBD_EINVAL;
  return guarded([&] { h->impl.zone_expand(active, n_rings); });
}

int mgpbd_mask_alpha(mgpbd_handle h, const int32_t* active, float* saved_alpha) {
  if (!h || !active || !saved_alpha) return MGPBD_EINVAL;
  return guarded([&] { h->impl.mask_alpha(active, saved_alpha); });
}

int mgpbd_restore_alpha(mgpbd_handle h, const float* saved_alpha) {
  if (!h || !saved_alpha) return MGPBD_EINVAL;
  return guarded([&] { h->impl.restore_alpha(saved_alpha); });
}

int mgpbd_level_sweep(mgpbd_handle h, int32_t level, int32_t op, const float* x, const float* b,
                      float* y, float omega) {
  if (!h || !x || !y || (op == 1 && !b)) return MGPBD_EINVAL;
  return guarded([&] { h->impl.level_sweep(level, op, x, b, y, omega); });
}

int mgpbd_synchronize(mgpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { MGPBD_CUDA(cudaStreamSynchronize(h->impl.stream())); });
}

// ---- standalone sparse kernels --------------------------------------------
int mgpbd_csr_spmv(int32_t n_rows, const int32_t* indptr, const int32_t* indices, const float* data,
                   const float* x, float* y, void* stream) {
  if (n_rows < 0 || (n_rows > 0 && (!indptr || !indices || !data || !x || !y))) return MGPBD_EINVAL;
  return guarded([&] {
    mgpbd::CsrView a;
    a.n = n_rows;
    int32_t nnz = 0;
    if (n_rows > 0)
      MGPBD_CUDA(cudaMemcpyAsync(&nnz, indptr + n_rows, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                 as_stream(stream)));
    MGPBD_CUDA(cudaStreamSynchronize(as_stream(stream)));
    a.nnz = nnz;
    a.indptr = indptr;
    a.indices = indices;
    a.data = data;
    mgpbd::launch_spmv(a, x, y, as_stream(stream));
  });
}

int mgpbd_csr_jacobi(int32_t n_rows, const int32_t* indptr, const int32_t* indices,
                     const float* data, const float* diag_inv, const float* b, const float* x,
                     float* x_new, float omega, void* stream) {
  if (n_rows < 0 || (n_rows > 0 && (!indptr || !indices || !data || !diag_inv || !b || !x || !x_new)))
    return MGPBD_EINVAL;
  return guarded([&] {
    mgpbd::CsrView a;
    a.n = n_rows;
    int32_t nnz = 0;
    if (n_rows > 0)
      MGPBD_CUDA(cudaMemcpyAsync(&nnz, indptr + n_rows, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                 as_stream(stream)));
    MGPBD_CUDA(cudaStreamSynchronize(as_stream(stream)));
    a.nnz = nnz;
    a.indptr = indptr;
    a.indices = indices;
    a.data = data;
    a.diag_inv = diag_inv;
    mgpbd::launch_jacobi(a, b, x, x_new, omega, as_stream(stream));
  });
}

int mgpbd_csr_diag_inv(int32_t n_rows, const int32_t* indptr, const int32_t* indices,
                       const float* data, float* diag_inv, void* stream) {
  if (n_rows < 0 || (n_rows > 0 && (!indptr || !indices || !data || !diag_inv))) return MGPBD_EINVAL;
  return guarded([&] { mgpbd::launch_diag_inv_scan(indptr, indices, data, n_rows, diag_inv, as_stream(stream)); });
}

int mgpbd_dot(int32_t n, const float* a, const float* b, double* out, void* stream) {
  if (n < 0 || !out || (n > 0 && (!a || !b))) return MGPBD_EINVAL;
  return guarded([&] {
    int blocks = mgpbd::reduce_blocks(n);
    mgpbd::DevBuf<double> part(blocks + 1);
    cudaStream_t s = as_stream(stream);
    mgpbd::launch_dot_partials(a, b, n, part.p, s);
    mgpbd::launch_finalize(part.p, blocks, 1, part.p + blocks, s);
    MGPBD_CUDA(cudaMemcpyAsync(out, part.p + blocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    MGPBD_CUDA(cudaStreamSynchronize(s));
  });
}

int mgpbd_axpy(int32_t n, float alpha, const float* x, float* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return MGPBD_EINVAL;
  return guarded([&] { mgpbd::launch_axpy(alpha, x, y, n, as_stream(stream)); });
}

int mgpbd_xpay(int32_t n, float alpha, const float* x, float* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return MGPBD_EINVAL;
  return guarded([&] { mgpbd::launch_xpay(alpha, x, y, n, as_stream(stream)); });
}

int mgpbd_scale(int32_t n, float alpha, float* x, void* stream) {
  if (n < 0 || (n > 0 && !x)) return MGPBD_EINVAL;
  return guarded([&] { mgpbd::launch_scale(alpha, x, n, as_stream(stream)); });
}

// ---- host structure builders ----------------------------------------------
int mgpbd_host_vertex_incidence(const int32_t* t_i, int32_t nt, int32_t nv, int64_t* n_entries,
                                int32_t* ptr, int32_t* entries) {
  if (!t_i || nt < 0 || nv < 0 || !n_entries) return MGPBD_EINVAL;
  return guarded([&] {
    for (int64_t k = 0; k < 4LL * nt; ++k)
      mgpbd::require(t_i[k] >= 0 && t_i[k] < nv, MGPBD_EINVAL, "vertex id out of range");
    std::vector<int32_t> p, e;
    mgpbd::vertex_incidence(t_i, nt, nv, p, e);
    *n_entries = static_cast<int64_t>(e.size());
    if (ptr) {
      mgpbd::require(entries != nullptr || e.empty(), MGPBD_EINVAL, "entries buffer missing");
      std::memcpy(ptr, p.data(), sizeof(int32_t) * p.size());
      if (!e.empty()) std::memcpy(entries, e.data(), sizeof(int32_t) * e.size());
    }
  });
}

int mgpbd_host_pattern(const int32_t* t_i, int32_t nt, int64_t* nnz, int32_t* indptr,
                       int32_t* indices) {
  if (!t_i || nt < 0 || !nnz) return MGPBD_EINVAL;
  return guarded([&] {
    mgpbd::Csr p = mgpbd::build_pattern(t_i, nt);
    *nnz = p.nnz();
    if (indptr) {
      mgpbd::require(indices != nullptr, MGPBD_EINVAL, "indices buffer missing");
      std::memcpy(indptr, p.indptr.data(), sizeof(int32_t) * p.indptr.size());
      std::memcpy(indices, p.indices.data(), sizeof(int32_t) * p.indices.size());
    }
  });
}

int mgpbd_host_aggregate(const int32_t* t_i, int32_t nt, int32_t max_agg_size, int32_t* agg_ids,
                         int32_t* n_agg) {
  if (!t_i || nt < 0 || !agg_ids || !n_agg || max_agg_size < 1) return MGPBD_EINVAL;
  return guarded([&] {
    std::vector<int32_t> a;
    *n_agg = mgpbd::tet_aggregate(t_i, nt, max_agg_size, a);
    std::memcpy(agg_ids, a.data(), sizeof(int32_t) * a.size());
  });
}

int mgpbd_host_tet_hierarchy(const int32_t* t_i, int32_t nt, int32_t max_coarse,
                             int32_t max_levels, int32_t* n_levels, int32_t* sizes,
                             int32_t* agg_ids) {
  if (!t_i || nt < 0 || !n_levels || !sizes || !agg_ids) return MGPBD_EINVAL;
  return guarded([&] {
    std::vector<int32_t> sz;
    std::vector<std::vector<int32_t>> aggs;
    mgpbd::tet_hierarchy(t_i, nt, max_coarse, max_levels, sz, aggs);
    *n_levels = static_cast<int32_t>(sz.size());
    std::memcpy(sizes, sz.data(), sizeof(int32_t) * sz.size());
    if (!aggs.empty()) std::memcpy(agg_ids, aggs[0].data(), sizeof(int32_t) * aggs[0].size());
  });
}

int mgpbd_host_face_adjacency(const int32_t* t_i, int32_t nt, int64_t* nnz, int32_t* indptr,
                              int32_t* indices) {
  if (!t_i || nt < 0 || !nnz) return MGPBD_EINVAL;
  return guarded([&] {
    mgpbd::Csr a = mgpbd::face_adjacency(t_i, nt);
    *nnz = a.nnz();
    if (indptr) std::copy(a.indptr.begin(), a.indptr.end(), indptr);
    if (indices) std::copy(a.indices.begin(), a.indices.end(), indices);
  });
}

int mgpbd_host_galerkin(int32_t n, const int32_t* indptr, const int32_t* indices, const float* data,
                        const int32_t* agg_ids, int32_t n_agg, int64_t* c_nnz, int64_t* n_contrib,
                        int32_t* c_indptr, int32_t* c_indices, int32_t* contrib_idx,
                        int32_t* contrib_off) {
  if (n < 0 || !indptr || !indices || !data || !agg_ids || n_agg < 0 || !c_nnz || !n_contrib)
    return MGPBD_EINVAL;
  return guarded([&] {
    mgpbd::Csr f;
    f.n_rows = f.n_cols = n;
    f.indptr.assign(indptr, indptr + n + 1);
    f.indices.assign(indices, indices + indptr[n]);
    mgpbd::Galerkin g = mgpbd::galerkin(f, data, agg_ids, n_agg);
    *c_nnz = g.coarse.nnz();
    *n_contrib = static_cast<int64_t>(g.contrib_idx.size());
    if (c_indptr) {
      mgpbd::require(c_indices && contrib_idx && contrib_off, MGPBD_EINVAL, "output buffer missing");
      std::memcpy(c_indptr, g.coarse.indptr.data(), sizeof(int32_t) * g.coarse.indptr.size());
      std::memcpy(c_indices, g.coarse.indices.data(), sizeof(int32_t) * g.coarse.indices.size());
      std::memcpy(contrib_idx, g.contrib_idx.data(), sizeof(int32_t) * g.contrib_idx.size());
      std::memcpy(contrib_off, g.contrib_off.data(), sizeof(int32_t) * g.contrib_off.size());
    }
  });
}

int mgpbd_device_galerkin(int32_t n, const int32_t* indptr, const int32_t* indices,
                          const float* data, const int32_t* agg_ids, int32_t n_agg,
                          int64_t* c_nnz, int64_t* n_contrib, int32_t* c_indptr,
                          int32_t* c_indices, int32_t* contrib_idx, int32_t* contrib_off,
                          int32_t* diag_pos) {
  if (n <= 0 || !indptr || !indices || !agg_ids || n_agg <= 0 || !c_nnz || !n_contrib)
    return MGPBD_EINVAL;
  return guarded([&] {
    using mgpbd::require;
    require(indptr[0] == 0, MGPBD_EINVAL, "indptr must start at 0");
    for (int32_t i = 0; i < n; ++i) {
      require(indptr[i + 1] >= indptr[i], MGPBD_EINVAL, "indptr must not decrease");
      for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k)
        require(indices[k] >= 0 && indices[k] < n, MGPBD_EINVAL, "column index outside [0, n)");
      require(agg_ids[i] >= 0 && agg_ids[i] < n_agg, MGPBD_EINVAL, "aggregate id out of range");
    }
    const int64_t nnz = indptr[n];
    require(nnz > 0, MGPBD_EINVAL, "empty matrix");
    std::vector<int32_t> mp(n_agg + 1, 0), mr(n);
    for (int32_t i = 0; i < n; ++i) mp[agg_ids[i] + 1]++;
    for (int32_t a = 0; a < n_agg; ++a) mp[a + 1] += mp[a];
    std::vector<int32_t> cur(mp.begin(), mp.end() - 1);
    for (int32_t i = 0; i < n; ++i) mr[cur[agg_ids[i]]++] = i;
    cudaStream_t s = nullptr;
    MGPBD_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{s};
    auto put = [&](auto& d, const auto* h, int64_t count) {
      d.alloc(std::max<int64_t>(count, 1));
      MGPBD_CUDA(cudaMemcpyAsync(d.p, h, sizeof(*h) * count, cudaMemcpyHostToDevice, s));
    };
    mgpbd::DevBuf<int32_t> d_ip, d_ix, d_agg, d_mp, d_mr;
    mgpbd::DevBuf<float> d_a;
    put(d_ip, indptr, n + 1LL);
    put(d_ix, indices, nnz);
    put(d_agg, agg_ids, n);
    put(d_mp, mp.data(), n_agg + 1LL);
    put(d_mr, mr.data(), n);
    if (data) put(d_a, data, nnz);
    mgpbd::DeviceGalerkin g;
    mgpbd::galerkin_device(n, nnz, d_ip.p, d_ix.p, data ? d_a.p : nullptr, d_agg.p, d_mp.p,
                           d_mr.p, n_agg, g, s);
    int32_t nmap = 0;
    MGPBD_CUDA(cudaMemcpyAsync(&nmap, g.contrib_off.p + g.nnz, sizeof(int32_t),
                               cudaMemcpyDeviceToHost, s));
    MGPBD_CUDA(cudaStreamSynchronize(s));
    *c_nnz = g.nnz;
    *n_contrib = nmap;
    if (c_indptr) {
      require(c_indices && contrib_idx && contrib_off, MGPBD_EINVAL, "output buffer missing");
      std::memcpy(c_indptr, g.host_indptr.data(), sizeof(int32_t) * (n_agg + 1LL));
      std::memcpy(c_indices, g.host_indices.data(), sizeof(int32_t) * g.nnz);
      MGPBD_CUDA(cudaMemcpyAsync(contrib_idx, g.contrib_idx.p, sizeof(int32_t) * nmap,
                                 cudaMemcpyDeviceToHost, s));
      MGPBD_CUDA(cudaMemcpyAsync(contrib_off, g.contrib_off.p, sizeof(int32_t) * (g.nnz + 1),
                                 cudaMemcpyDeviceToHost, s));
      if (diag_pos)
        MGPBD_CUDA(cudaMemcpyAsync(diag_pos, g.diag_pos.p, sizeof(int32_t) * n_agg,
                                   cudaMemcpyDeviceToHost, s));
      MGPBD_CUDA(cudaStreamSynchronize(s));
    }
  });
}

// ---- comparison solvers (include/mgpbd_local.h) ----------------------------

int mgpbd_color_elements(const int32_t* elems, int32_t n_elements, int32_t verts_per_element,
                         int32_t n_vertices, int32_t* ordered, int32_t* offsets,
                         int32_t* n_colors) {
  if (!ordered || !offsets || !n_colors) return MGPBD_EINVAL;
  return guarded([&] {
    put_coloring(mgpbd::color_elements(elems, n_elements, verts_per_element, n_vertices), ordered,
                 offsets, n_colors);
  });
}

int mgpbd_color_vertices(const int32_t* elems, int32_t n_elements, int32_t verts_per_element,
                         int32_t n_vertices, int32_t* ordered, int32_t* offsets,
                         int32_t* n_colors) {
  if (!ordered || !offsets || !n_colors) return MGPBD_EINVAL;
  return guarded([&] {
    put_coloring(mgpbd::color_vertices(elems, n_elements, verts_per_element, n_vertices), ordered,
                 offsets, n_colors);
  });
}

int mgpbd_greedy_coloring(const int32_t* adj_ptr, const int32_t* adj, int32_t n,
                          int32_t* ordered, int32_t* offsets, int32_t* n_colors) {
  if (!ordered || !offsets || !n_colors) return MGPBD_EINVAL;
  return guarded(
      [&] { put_coloring(mgpbd::greedy_coloring_csr(adj_ptr, adj, n), ordered, offsets, n_colors); });
}

int mgpbd_xpbd_create(const mgpbd_xpbd_params* params, mgpbd_xpbd_handle* out) {
  if (!params || !out) return MGPBD_EINVAL;
  *out = nullptr;
  return guarded([&] { *out = new mgpbd_xpbd(*params); });
}

void mgpbd_xpbd_destroy(mgpbd_xpbd_handle h) { delete h; }

int mgpbd_xpbd_set_stream(mgpbd_xpbd_handle h, void* stream) {
  if (!h) return MGPBD_EINVAL;
  h->impl.set_stream(as_stream(stream));
  return MGPBD_OK;
}

int mgpbd_xpbd_set_mesh(mgpbd_xpbd_handle h, float* x, const float* x_ref, const float* invm,
                        const int32_t* t_i, const float* t_m, int32_t nv, int32_t nt) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_mesh(x, x_ref, invm, t_i, t_m, nv, nt); });
}

int mgpbd_xpbd_preupdate(mgpbd_xpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.preupdate(); });
}

int mgpbd_xpbd_update(mgpbd_xpbd_handle h, int32_t n_passes) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.update(n_passes); });
}

int mgpbd_xpbd_synchronize(mgpbd_xpbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.synchronize(); });
}

int mgpbd_xpbd_lambdas(mgpbd_xpbd_handle h, float** hydro, float** devia) {
  if (!h || !hydro || !devia) return MGPBD_EINVAL;
  *hydro = h->impl.lambda_h();
  *devia = h->impl.lambda_d();
  return *hydro ? MGPBD_OK : MGPBD_ESTATE;
}

int mgpbd_xpbd_n_colors(mgpbd_xpbd_handle h, int32_t* n_colors) {
  if (!h || !n_colors) return MGPBD_EINVAL;
  *n_colors = h->impl.n_colors();
  return MGPBD_OK;
}

int mgpbd_vbd_create(const mgpbd_vbd_params* params, mgpbd_vbd_handle* out) {
  if (!params || !out) return MGPBD_EINVAL;
  *out = nullptr;
  return guarded([&] { *out = new mgpbd_vbd(*params); });
}

void mgpbd_vbd_destroy(mgpbd_vbd_handle h) { delete h; }

int mgpbd_vbd_set_stream(mgpbd_vbd_handle h, void* stream) {
  if (!h) return MGPBD_EINVAL;
  h->impl.set_stream(as_stream(stream));
  return MGPBD_OK;
}

int mgpbd_vbd_set_mesh(mgpbd_vbd_handle h, float* x, const float* x_ref, const float* invm,
                       const int32_t* t_i, int32_t nv, int32_t nt) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.set_mesh(x, x_ref, invm, t_i, nv, nt); });
}

int mgpbd_vbd_init(mgpbd_vbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.init(); });
}

int mgpbd_vbd_make_prediction(mgpbd_vbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.make_prediction(); });
}

int mgpbd_vbd_solve(mgpbd_vbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.solve(); });
}

int mgpbd_vbd_update_vel(mgpbd_vbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.update_vel(); });
}

int mgpbd_vbd_step(mgpbd_vbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.step(); });
}

int mgpbd_vbd_synchronize(mgpbd_vbd_handle h) {
  if (!h) return MGPBD_EINVAL;
  return guarded([&] { h->impl.synchronize(); });
}

int mgpbd_vbd_omegas(mgpbd_vbd_handle h, float* omegas) {
  if (!h || !omegas) return MGPBD_EINVAL;
  const auto& o = h->impl.omegas();
  std::copy(o.begin(), o.end(), omegas);
  return MGPBD_OK;
}

int mgpbd_vbd_field(mgpbd_vbd_handle h, int32_t field, void** dev_ptr, int64_t* count) {
  if (!h || !dev_ptr || !count) return MGPBD_EINVAL;
  return guarded([&] {
    *dev_ptr = h->impl.field(field, count);
    mgpbd::require(*dev_ptr != nullptr, MGPBD_ESTATE, "vbd: set_mesh has not been called");
  });
}

int mgpbd_vbd_n_colors(mgpbd_vbd_handle h, int32_t* n_colors) {
  if (!h || !n_colors) return MGPBD_EINVAL;
  *n_colors = h->impl.n_colors();
  return MGPBD_OK;
}

int mgpbd_vbd_lame(mgpbd_vbd_handle h, float* mu, float* lam) {
  if (!h || !mu || !lam) return MGPBD_EINVAL;
  *mu = h->impl.mu();
  *lam = h->impl.lam();
  return MGPBD_OK;
}

}  // extern "C"
