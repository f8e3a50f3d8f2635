// mgpbd_dot_noalloc: the float64 dot product of mgpbd_dot with its scratch
// in a fixed device array instead of a per-call cudaMalloc.
//
// Who needs it: a host application that embeds this library but owns the
// GPU memory budget (a game engine, a DCC-tool plugin host, a real-time
// loop with a fixed memory plan) may forbid its plugins from calling
// cudaMalloc/cudaFree: those calls can block until the device is idle,
// which stalls the caller's other streams mid-frame, and they bypass the
// host's allocator and accounting.  Such a caller passes its own input
// buffers and this entry point touches no other memory than the array
// below, which every GPU that loads the library holds until the process
// exits.
#include <cuda_runtime.h>

#include <mutex>

#include "common.h"

namespace mgpbd {
namespace {

// One float64 partial sum per 1024 input elements, plus the result slot.
constexpr int kNaThreads = 256;
constexpr int kNaPerBlock = 1024;  // elements per partial sum
constexpr int64_t kNaMaxPartials = 65536;
constexpr int64_t kNaMaxN = kNaMaxPartials * kNaPerBlock;  // 67,108,864 elements
// 512 KiB + the result slot; a host-side name only, never dereferenced on
// the host: kernels get the device address from cudaGetSymbolAddress.
__device__ __align__(256) double g_dot_scratch[kNaMaxPartials + 32];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

// Device address of the scratch array for the current device, looked up
// once per device (with that device current) and cached.
double* scratch_address() {
  int dev = 0;
  MGPBD_CUDA(cudaGetDevice(&dev));
  require(dev >= 0 && dev < kMaxDevices, MGPBD_ERANGE, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dot_scratch);
    if (e != cudaSuccess)
      throw Error(MGPBD_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<double*>(p);
  }
  return g_addr[dev];
}

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double na_block_sum(double v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = na_warp_sum(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) v = na_warp_sum(v);
  __syncthreads();
  return v;
}

// block b sums elements [1024 b, 1024 (b + 1)) in a fixed order
__global__ void k_na_partials(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                              double* __restrict__ partials) {
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kNaPerBlock;
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < kNaPerBlock / kNaThreads; ++k) {
    const int64_t i = base + k * kNaThreads + threadIdx.x;
    if (i < n) acc += static_cast<double>(a[i]) * static_cast<double>(b[i]);
  }
  acc = na_block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void k_na_final(const double* __restrict__ partials, int64_t nb, double* __restrict__ out) {
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[i];
  acc = na_block_sum(acc);
  if (threadIdx.x == 0) *out = acc;
}

}  // namespace
}  // namespace mgpbd

extern "C" int mgpbd_dot_noalloc(int32_t n, const float* a, const float* b, double* out,
                                 void* stream) {
  if (n < 0 || !out || (n > 0 && (!a || !b))) {
    mgpbd::set_last_error("mgpbd_dot_noalloc: n < 0 or a null pointer");
    return MGPBD_EINVAL;
  }
  if (static_cast<int64_t>(n) > mgpbd::kNaMaxN) {
    mgpbd::set_last_error("mgpbd_dot_noalloc: n above 67,108,864 (the fixed scratch holds one "
                          "partial sum per 1024 elements, 65,536 at most)");
    return MGPBD_ERANGE;
  }
  try {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double* scratch = mgpbd::scratch_address();
    double* result = scratch + mgpbd::kNaMaxPartials;
    const int64_t nb = (static_cast<int64_t>(n) + mgpbd::kNaPerBlock - 1) / mgpbd::kNaPerBlock;
    if (nb > 0) {
      mgpbd::k_na_partials<<<static_cast<unsigned>(nb), mgpbd::kNaThreads, 0, s>>>(a, b, n, scratch);
      MGPBD_CHECK_LAUNCH();
    }
    // n == 0 sums no partials and writes 0: the slot keeps nothing of the
    // previous call
    mgpbd::k_na_final<<<1, mgpbd::kNaThreads, 0, s>>>(scratch, nb, result);
    MGPBD_CHECK_LAUNCH();
    MGPBD_CUDA(cudaMemcpyAsync(out, result, sizeof(double), cudaMemcpyDeviceToHost, s));
    MGPBD_CUDA(cudaStreamSynchronize(s));
    return MGPBD_OK;
  } catch (const mgpbd::Error& e) {
    mgpbd::set_last_error(std::string("mgpbd_dot_noalloc: ") + e.what());
    return e.code;
  } catch (const std::exception& e) {
    mgpbd::set_last_error(std::string("mgpbd_dot_noalloc: ") + e.what());
    return MGPBD_EINVAL;
  }
}
