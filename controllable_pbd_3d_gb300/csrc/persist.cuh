// Device helpers of the cooperative persistent CG kernels (jcg.cu, pcg.cu):
// the bounded grid barrier and the fixed-order block/grid reductions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mgpbd.h"
#include "jform.cuh"
#include "jform_dev.cuh"

namespace mgpbd {
namespace pdev {

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long atom_add_acq_rel(unsigned long long* p,
                                                            unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;"
               : "=l"(old)
               : "l"(p), "l"(v)
               : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Grid-wide barrier over a monotonic arrival counter (barrier n of a launch
// completes when the counter reaches n * gridDim.x).  Thread 0 arrives with
// an acquire-release add after the block's bar.sync (so the block's writes
// are released), polls with relaxed loads and ends with an acquire fence
// before the closing bar.sync; the block that arrives last skips the poll.
// Returns false in all threads of the block if the wait gave up (limit
// reached, or another block gave up; spin_ns = 0 gives up at once when
// another block has not arrived yet); the failure is recorded in gs->err
// and as MGPBD_STATUS_SYNC_TIMEOUT in *status_word.
__device__ __forceinline__ bool grid_sync(GridSync* gs, int32_t* status_word,
                                          unsigned long long spin_ns, unsigned long long& gen) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    gen += 1;
    const unsigned long long target = gen * gridDim.x;
    const unsigned long long old = atom_add_acq_rel(&gs->count, 1ull);
    int ok = 1;
    if (old + 1 < target) {
      const unsigned long long t0 = global_ns();
      unsigned int n = 0;
      while (ld_relaxed(&gs->count) < target) {
        // the limit is checked every 64 polls; a limit of 0 gives up at the
        // first poll that finds the barrier incomplete
        if ((++n & 63u) == 0 || spin_ns == 0) {
          if (ld_relaxed(&gs->err) != 0u || global_ns() - t0 > spin_ns) {
            ok = 0;
            break;
          }
        }
      }
      fence_acq_rel();
    }
    if (!ok) {
      atomicExch(&gs->err, 1u);
      atomicOr(reinterpret_cast<unsigned int*>(status_word), MGPBD_STATUS_SYNC_TIMEOUT);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Fixed-order float64 sum of n block partials by warp 0 (lane-strided
// chains, then a fixed shuffle tree), valid in lane 0.  The scalar logic
// that follows runs in thread 0 only: GB300's float64 rate is low, and the
// same arithmetic in every thread of every block saturates the pipe.
__device__ __forceinline__ double warp_sum_partials(const double* part, int n) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 32) acc += __ldcg(part + i);
  return jdev::warp_sum_d(acc);
}

__device__ __forceinline__ void put_partial(float v, double* slot) {
  const double s = jdev::block_sum_fd(v);
  if (threadIdx.x == 0) slot[blockIdx.x] = s;
}

}  // namespace pdev
}  // namespace mgpbd
