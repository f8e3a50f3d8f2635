// Galerkin coarse level built on the GPU (rap.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.h"
#include "kernels.cuh"

namespace mgpbd {

// The coarse level of (P^T A) P for P given by agg (fine row -> aggregate)
// and its members (mem_ptr / mem_rows, ascending within each aggregate):
// sorted coarse columns with exact float64 zeros dropped (none dropped when
// data is null: structural), the diagonal positions, and the contribution
// map (per coarse entry, the fine positions in member-ascending, stored
// order).  Bit-identical to the host builder `galerkin` /
// `galerkin_structural` (structure.h).  Device inputs; device outputs, with
// host copies of the coarse pattern.
struct DeviceGalerkin {
  DevBuf<int32_t> indptr, indices, contrib_off, contrib_idx, diag_pos;
  std::vector<int32_t> host_indptr, host_indices;
  int64_t nnz = 0;
};
void galerkin_device(int32_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                     const float* data, const int32_t* agg, const int32_t* mem_ptr,
                     const int32_t* mem_rows, int32_t n_agg, DeviceGalerkin& out,
                     cudaStream_t s);

}  // namespace mgpbd
