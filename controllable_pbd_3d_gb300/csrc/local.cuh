// Comparison solvers of the MGPBD convergence experiments: local XPBD
// (cons/deform3d.py) and Vertex Block Descent (cons/vbd.py).  The colour
// methods run as one cooperative kernel per pass / solve with a bounded grid
// barrier between colours; the serial methods keep the reference's order
// (one tet, or one vertex, at a time).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/mgpbd_local.h"
#include "common.h"
#include "jform.cuh"

namespace mgpbd {

// Status word of the cooperative colour kernels, read without stalling the
// stream: each launch queues a copy into pinned host memory and an event;
// the next call checks the copy if the event has completed (a grid barrier
// that gave up is reported then, as MGPBD_ECUDA).
class LazyStatus {
 public:
  LazyStatus() = default;
  LazyStatus(const LazyStatus&) = delete;
  LazyStatus& operator=(const LazyStatus&) = delete;
  ~LazyStatus();
  void record(const int32_t* dev, cudaStream_t s);
  void check(const char* what);
  void wait(const char* what);

 private:
  int32_t* host_ = nullptr;
  cudaEvent_t ev_ = nullptr;
  bool pending_ = false;
};

class Xpbd {
 public:
  explicit Xpbd(const mgpbd_xpbd_params& p);
  void set_stream(cudaStream_t s) { stream_ = s; }
  void set_mesh(float* x, const float* x_ref, const float* invm, const int32_t* t_i,
                const float* t_m, int32_t nv, int32_t nt);
  void preupdate();
  void update(int32_t passes);
  void synchronize() { lazy_.wait("xpbd colour kernel"); }
  float* lambda_h() const { return lam_h_.p; }
  float* lambda_d() const { return lam_d_.p; }
  int32_t n_colors() const { return n_colors_; }

 private:
  mgpbd_xpbd_params p_;
  LazyStatus lazy_;
  cudaStream_t stream_ = nullptr;
  float* x_ = nullptr;
  const float* invm_ = nullptr;
  const float* t_m_ = nullptr;
  const int32_t* t_i_ = nullptr;
  int32_t nv_ = 0, nt_ = 0;
  DevBuf<float> B_, lam_h_, lam_d_;
  DevBuf<int32_t> order_, offsets_, status_;
  DevBuf<GridSync> gs_;
  int32_t n_colors_ = 0;
  int grid_ = 0;
};

class Vbd {
 public:
  explicit Vbd(const mgpbd_vbd_params& p);
  void set_stream(cudaStream_t s) { stream_ = s; }
  void set_mesh(float* x, const float* x_ref, const float* invm, const int32_t* t_i, int32_t nv,
                int32_t nt);
  void init();
  void make_prediction();
  void solve();
  void update_vel();
  void synchronize() { lazy_.wait("vbd colour kernel"); }
  void step() {
    make_prediction();
    solve();
    update_vel();
  }
  const std::vector<float>& omegas() const { return omegas_; }
  void* field(int32_t f, int64_t* count);
  int32_t n_colors() const { return n_colors_; }
  float mu() const { return mu_; }
  float lam() const { return lam_; }

 private:
  mgpbd_vbd_params p_;
  LazyStatus lazy_;
  float mu_ = 0.0f, lam_ = 0.0f;
  std::vector<float> omegas_;
  cudaStream_t stream_ = nullptr;
  float* x_ = nullptr;
  const float* x_ref_ = nullptr;
  const float* invm_ = nullptr;
  const int32_t* t_i_ = nullptr;
  int32_t nv_ = 0, nt_ = 0;
  bool inited_ = false;
  DevBuf<float> v_, x_old_, x_tilde_, x_prev_, dm_inv_, vol_, om_;
  DevBuf<int32_t> adj_ptr_, adj_, order_, offsets_, status_;
  DevBuf<GridSync> gs_;
  int32_t n_colors_ = 0;
  int grid_ = 0;
};

}  // namespace mgpbd
