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

class Xpbd {
 public:
  explicit Xpbd(const mgpbd_xpbd_params& p);
  void set_stream(cudaStream_t s) { stream_ = s; }
  void set_mesh(float* x, const float* x_ref, const float* invm, const int32_t* t_i,
                const float* t_m, int32_t nv, int32_t nt);
  void preupdate();
  void update(int32_t passes);
  float* lambda_h() const { return lam_h_.p; }
  float* lambda_d() const { return lam_d_.p; }
  int32_t n_colors() const { return n_colors_; }

 private:
  void check_status();
  mgpbd_xpbd_params p_;
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
  void check_status();
  mgpbd_vbd_params p_;
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
