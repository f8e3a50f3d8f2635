// Shared definitions for the MGPBD CUDA library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/mgpbd.h"

namespace mgpbd {

// Exceptions never cross the C ABI; capi.cu maps them to MGPBD_E* codes.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A failed call also leaves its error as the runtime's "last error"; it is
// read back (cleared) here so the next launch check does not report it
// again (sticky errors of a lost context stay, as they must).
#define MGPBD_CUDA(call)                                                           \
  do {                                                                             \
    cudaError_t err_ = (call);                                                     \
    if (err_ != cudaSuccess) {                                                     \
      (void)cudaGetLastError();                                                    \
      throw ::mgpbd::Error(MGPBD_ECUDA, std::string(#call) + ": " +                \
                                            cudaGetErrorString(err_));             \
    }                                                                              \
  } while (0)

// Every kernel launch of the library goes through this macro, which also
// counts it (mgpbd_launch_count).  Launches recorded into a CUDA graph are
// counted when the graph runs (see Solver::pcg_graph).
extern std::atomic<long long> g_launches;
#define MGPBD_CHECK_LAUNCH()                                  \
  do {                                                        \
    ::mgpbd::g_launches.fetch_add(1, std::memory_order_relaxed); \
    MGPBD_CUDA(cudaGetLastError());                           \
  } while (0)

inline void require(bool ok, int code, const char* msg) {
  if (!ok) throw Error(code, msg);
}

// Records the message that mgpbd_last_error() returns on the calling
// thread (defined in capi.cu beside the C ABI's error mapping).
void set_last_error(const std::string& msg);

// Owning device buffer (cudaMalloc / cudaFree).
template <class T>
struct DevBuf {
  T* p = nullptr;
  int64_t n = 0;
  DevBuf() = default;
  explicit DevBuf(int64_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(int64_t count) {
    release();
    n = count;
    if (count > 0) {
      cudaError_t e = cudaMalloc(&p, sizeof(T) * static_cast<size_t>(count));
      if (e != cudaSuccess) {
        p = nullptr;
        n = 0;
        throw Error(MGPBD_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
      }
    }
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  T* get() const { return p; }
};

inline int ceil_div(int64_t a, int64_t b) { return static_cast<int>((a + b - 1) / b); }

}  // namespace mgpbd
