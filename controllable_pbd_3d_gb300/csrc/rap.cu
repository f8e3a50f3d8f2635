// Galerkin coarse level of an aggregation prolongation built on the GPU:
// the pattern of (P^T A) P with exact-zero dropping and the contribution map
// that GPUMultigridSolver.setup computes on the host (cons/mgpcg_gpu.py:
// 43-99), bit-identical to the host builder `galerkin` (structure.cpp).
//
// One warp per coarse row I.  Its fine rows (the aggregate's members, in
// ascending order) are walked entry by entry; a hash table of the row's
// fine columns j (open addressing in a per-row slice of global scratch)
// accumulates X[I, j] = sum over members of A[i, j] in float64, in member
// order, as the host does.  The coarse columns J are the aggregates of the
// touched j with X != 0, ranked into ascending order, and each is summed
// as sum over j in J (ascending, members of J) of X[I, j], again the host's
// order, so the exact zeros dropped are the same.  A second pass lists,
// per kept (I, J), the fine positions in (member ascending, stored
// position) order.
#include <cuda_runtime.h>

#include <algorithm>

#include "rap.cuh"

namespace mgpbd {
namespace {

constexpr int kRapWarps = 8;  // warps per block, one coarse row each

__device__ __forceinline__ uint32_t rap_hash(int32_t j) {
  return static_cast<uint32_t>(j) * 2654435761u;
}

// slot of key j in the table [keys, keys + cap) (cap a power of two), or
// -1 if absent
__device__ __forceinline__ int64_t rap_find(const int32_t* keys, int64_t cap, int32_t j) {
  int64_t s = rap_hash(j) & (cap - 1);
  for (int64_t probe = 0; probe < cap; ++probe) {
    const int32_t k = keys[s];
    if (k == j) return s;
    if (k < 0) return -1;
    s = (s + 1) & (cap - 1);
  }
  return -1;
}

// per coarse row: the fine entries of its members (len) and its table
// capacity (a power of two >= 2 len, at least 32)
__global__ void k_rap_len(const int32_t* __restrict__ indptr, const int32_t* __restrict__ mem_ptr,
                          const int32_t* __restrict__ mem_rows, int32_t n_agg,
                          int64_t* __restrict__ cap) {
  const int32_t I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n_agg) return;
  int64_t len = 0;
  for (int32_t m = mem_ptr[I]; m < mem_ptr[I + 1]; ++m) {
    const int32_t i = mem_rows[m];
    len += indptr[i + 1] - indptr[i];
  }
  int64_t c = 32;
  while (c < 2 * len) c <<= 1;
  cap[I] = c;
}

// ---- exclusive scan (setup sizes: a few million entries) -------------------
// out[0..n] = 0, in[0], in[0] + in[1], ...: blocks of kScanItems scanned
// locally with their totals in sums, the totals scanned by one block, then
// added back.
constexpr int kScanThreads = 256, kScanPer = 4, kScanItems = kScanThreads * kScanPer;

// exclusive scan of v over a block of kScanThreads threads (sh: 32 entries);
// returns the thread's offset, *total the block's sum
template <class T>
__device__ T block_exclusive(T v, T* sh, T* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T inc = v;
  for (int d = 1; d < 32; d <<= 1) {
    const T u = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += u;
  }
  if (lane == 31) sh[w] = inc;
  __syncthreads();
  if (w == 0) {
    T x = lane < nw ? sh[lane] : T(0);
    for (int d = 1; d < 32; d <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += u;
    }
    if (lane < nw) sh[lane] = x;  // inclusive warp totals
  }
  __syncthreads();
  const T before = w > 0 ? sh[w - 1] : T(0);
  *total = sh[nw - 1];
  __syncthreads();  // sh reused by the next call
  return before + inc - v;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads)
    k_scan_blocks(const T* __restrict__ in, int64_t n, T* __restrict__ out, T* __restrict__ sums) {
  __shared__ T sh[32];
  const int64_t base = blockIdx.x * static_cast<int64_t>(kScanItems) + threadIdx.x * kScanPer;
  T v[kScanPer], t = 0;
  for (int q = 0; q < kScanPer; ++q) {
    v[q] = base + q < n ? in[base + q] : T(0);
    t += v[q];
  }
  T total;
  T run = block_exclusive(t, sh, &total);
  for (int q = 0; q < kScanPer; ++q) {
    if (base + q < n) out[base + q] = run;
    run += v[q];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// one block: sums[b] <- exclusive scan, out[n] <- the grand total
template <class T>
__global__ void __launch_bounds__(1024) k_scan_sums(T* __restrict__ sums, int64_t nb,
                                                    T* __restrict__ last) {
  __shared__ T sh[32];
  T carry = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    const int64_t b = b0 + threadIdx.x;
    const T v = b < nb ? sums[b] : T(0);
    T total;
    const T e = block_exclusive(v, sh, &total);
    if (b < nb) sums[b] = carry + e;
    carry += total;
  }
  if (threadIdx.x == 0) *last = carry;
}

template <class T>
__global__ void k_scan_add(T* __restrict__ out, int64_t n, const T* __restrict__ sums) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[i] += sums[i / kScanItems];
}

// out (n + 1 entries) = exclusive scan of in (n entries)
template <class T>
void exclusive_scan(const T* in, int64_t n, T* out, cudaStream_t s) {
  const int64_t nb = std::max<int64_t>(1, (n + kScanItems - 1) / kScanItems);
  DevBuf<T> sums;
  sums.alloc(nb);
  k_scan_blocks<T><<<static_cast<unsigned>(nb), kScanThreads, 0, s>>>(in, n, out, sums.p);
  MGPBD_CHECK_LAUNCH();
  k_scan_sums<T><<<1, 1024, 0, s>>>(sums.p, nb, out + n);
  MGPBD_CHECK_LAUNCH();
  k_scan_add<T><<<static_cast<unsigned>(std::min<int64_t>(nb * 4, 4096)), 256, 0, s>>>(out, n,
                                                                                      sums.p);
  MGPBD_CHECK_LAUNCH();
  MGPBD_CUDA(cudaStreamSynchronize(s));  // sums is freed on return
}

// X[I, j] by member rows in order; candidates J ranked ascending (through
// the row's slice of `sorted`); kept columns (acc != 0, or all when
// structural) written to cols from the start of the row's slice, their
// count to row_nnz[I]
__global__ void __launch_bounds__(32 * kRapWarps)
    k_rap_rows(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
               const float* __restrict__ data, const int32_t* __restrict__ agg,
               const int32_t* __restrict__ mem_ptr, const int32_t* __restrict__ mem_rows,
               int32_t n_agg, const int64_t* __restrict__ off, int32_t* __restrict__ keys,
               double* __restrict__ vals, int32_t* __restrict__ cols,
               int32_t* __restrict__ sorted, int32_t* __restrict__ row_nnz,
               int32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int32_t I = blockIdx.x * kRapWarps + (threadIdx.x >> 5);
  if (I >= n_agg) return;
  const int64_t o = off[I], cap = off[I + 1] - o;
  int32_t* K = keys + o;
  double* V = vals + o;
  int32_t* Jl = cols + o;  // candidate / kept coarse columns of this row
  // stage 1: X[I, j] += A[i, j] for members i ascending, stored positions
  // ascending; the lanes of a chunk holding the same j (a repeated column)
  // leave the adds to the first of them, which makes them in lane order
  for (int32_t m = mem_ptr[I]; m < mem_ptr[I + 1]; ++m) {
    const int32_t i = mem_rows[m];
    const int32_t end = indptr[i + 1];
    for (int32_t k0 = indptr[i]; k0 < end; k0 += 32) {
      const int32_t k = k0 + lane;
      const int32_t j = k < end ? indices[k] : -1 - lane;
      const unsigned grp = __match_any_sync(0xffffffffu, j);
      if (k < end && (__ffs(grp) - 1) == lane) {
        int64_t s = rap_hash(j) & (cap - 1);
        int64_t probe = 0;
        for (; probe < cap; ++probe) {
          const int32_t prev = atomicCAS(K + s, -1, j);
          if (prev == -1 || prev == j) break;
          s = (s + 1) & (cap - 1);
        }
        if (probe == cap) {
          atomicExch(err, 1);
        } else if (data) {
          for (unsigned g = grp; g; g &= g - 1)
            V[s] += static_cast<double>(data[k0 + __ffs(g) - 1]);
        }
      }
      __syncwarp();
    }
  }
  // candidate coarse columns: aggregates of the touched j with X != 0, each
  // once (the lane that finds J first in slot order claims it)
  int32_t nc = 0;
  for (int64_t s0 = 0; s0 < cap; s0 += 32) {
    const int64_t s = s0 + lane;
    int32_t J = -1;
    if (s < cap && K[s] >= 0 && (!data || V[s] != 0.0)) J = agg[K[s]];
    // drop J already listed, or held by a lower lane of this chunk
    bool fresh = J >= 0;
    for (int32_t c = 0; c < nc && fresh; ++c) fresh = Jl[c] != J;
    const unsigned same = __match_any_sync(0xffffffffu, fresh ? J : -1 - lane);
    fresh = fresh && (__ffs(same) - 1) == lane;
    const unsigned take = __ballot_sync(0xffffffffu, fresh);
    if (fresh) Jl[nc + __popc(take & ((1u << lane) - 1))] = J;
    nc += __popc(take);
    __syncwarp();
  }
  // ascending order: a candidate's rank among the (distinct) candidates is
  // its place in St
  int32_t* St = sorted + o;
  for (int32_t c = lane; c < nc; c += 32) {
    const int32_t J = Jl[c];
    int32_t rank = 0;
    for (int32_t d = 0; d < nc; ++d) rank += Jl[d] < J;
    St[rank] = J;
  }
  __syncwarp();
  // per candidate J: sum over its members j ascending of X[I, j]; kept if
  // non-zero (structural: always); the kept columns compacted into Jl in
  // ascending order
  int32_t nk = 0;
  for (int32_t c0 = 0; c0 < nc; c0 += 32) {
    const int32_t c = c0 + lane;
    bool kp = false;
    int32_t J = 0;
    if (c < nc) {
      J = St[c];
      kp = true;
      if (data) {
        double acc = 0.0;
        for (int32_t mm = mem_ptr[J]; mm < mem_ptr[J + 1]; ++mm) {
          const int64_t s = rap_find(K, cap, mem_rows[mm]);
          if (s >= 0) {
            const double x = V[s];
            if (x != 0.0) acc += x;
          }
        }
        kp = acc != 0.0;
      }
    }
    const unsigned take = __ballot_sync(0xffffffffu, kp);
    if (kp) Jl[nk + __popc(take & ((1u << lane) - 1))] = J;
    nk += __popc(take);
  }
  if (lane == 0) row_nnz[I] = nk;
}

// coarse columns into place, the diagonal position, and the number of
// fine entries per kept coarse entry
__global__ void __launch_bounds__(32 * kRapWarps)
    k_rap_place(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                const int32_t* __restrict__ agg, const int32_t* __restrict__ mem_ptr,
                const int32_t* __restrict__ mem_rows, int32_t n_agg,
                const int64_t* __restrict__ off, const int32_t* __restrict__ cols,
                const int32_t* __restrict__ c_indptr, int32_t* __restrict__ c_indices,
                int32_t* __restrict__ diag_pos, int32_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int32_t I = blockIdx.x * kRapWarps + (threadIdx.x >> 5);
  if (I >= n_agg) return;
  const int32_t* Jl = cols + off[I];
  const int32_t b = c_indptr[I], nk = c_indptr[I + 1] - b;
  for (int32_t c = lane; c < nk; c += 32) {
    c_indices[b + c] = Jl[c];
    if (Jl[c] == I) diag_pos[I] = b + c;
  }
  for (int32_t m = mem_ptr[I]; m < mem_ptr[I + 1]; ++m) {
    const int32_t i = mem_rows[m];
    for (int32_t k = indptr[i] + lane; k < indptr[i + 1]; k += 32) {
      const int32_t J = agg[indices[k]];
      int32_t lo = 0, hi = nk;  // kept columns are ascending
      while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (Jl[mid] < J) lo = mid + 1;
        else hi = mid;
      }
      if (lo < nk && Jl[lo] == J) atomicAdd(cnt + b + lo, 1);
    }
  }
}

// the contribution map: per kept (I, J), the fine positions in (member
// ascending, stored position) order
__global__ void __launch_bounds__(32 * kRapWarps)
    k_rap_map(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
              const int32_t* __restrict__ agg, const int32_t* __restrict__ mem_ptr,
              const int32_t* __restrict__ mem_rows, int32_t n_agg,
              const int32_t* __restrict__ c_indptr, const int32_t* __restrict__ c_indices,
              const int32_t* __restrict__ c_off, int32_t* __restrict__ cursor,
              int32_t* __restrict__ c_idx) {
  const int lane = threadIdx.x & 31;
  const int32_t I = blockIdx.x * kRapWarps + (threadIdx.x >> 5);
  if (I >= n_agg) return;
  const int32_t b = c_indptr[I], nk = c_indptr[I + 1] - b;
  const int32_t* Jl = c_indices + b;
  for (int32_t m = mem_ptr[I]; m < mem_ptr[I + 1]; ++m) {
    const int32_t i = mem_rows[m];
    for (int32_t k0 = indptr[i]; k0 < indptr[i + 1]; k0 += 32) {
      const int32_t k = k0 + lane;
      int32_t c = -1;
      if (k < indptr[i + 1]) {
        const int32_t J = agg[indices[k]];
        int32_t lo = 0, hi = nk;
        while (lo < hi) {
          const int32_t mid = (lo + hi) >> 1;
          if (Jl[mid] < J) lo = mid + 1;
          else hi = mid;
        }
        if (lo < nk && Jl[lo] == J) c = b + lo;
      }
      // lanes of one coarse entry append in lane (= stored position) order
      const unsigned grp = __match_any_sync(0xffffffffu, c >= 0 ? c : -2 - lane);
      if (c >= 0) {
        const int32_t base = cursor[c];
        const int rank = __popc(grp & ((1u << lane) - 1));
        c_idx[c_off[c] + base + rank] = k;
      }
      __syncwarp();
      if (c >= 0 && (__ffs(grp) - 1) == lane) cursor[c] += __popc(grp);
      __syncwarp();
    }
  }
}

}  // namespace

void galerkin_device(int32_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                     const float* data, const int32_t* agg, const int32_t* mem_ptr,
                     const int32_t* mem_rows, int32_t n_agg, DeviceGalerkin& out,
                     cudaStream_t s) {
  require(n > 0 && n_agg > 0 && nnz > 0, MGPBD_EINVAL, "device Galerkin: empty level");
  const int rb = (n_agg + kRapWarps - 1) / kRapWarps;
  DevBuf<int64_t> cap, off;
  cap.alloc(n_agg);
  off.alloc(static_cast<int64_t>(n_agg) + 1);
  k_rap_len<<<(n_agg + 255) / 256, 256, 0, s>>>(indptr, mem_ptr, mem_rows, n_agg, cap.p);
  MGPBD_CHECK_LAUNCH();
  exclusive_scan(cap.p, n_agg, off.p, s);
  int64_t total = 0;
  MGPBD_CUDA(cudaMemcpyAsync(&total, off.p + n_agg, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
  DevBuf<int32_t> keys, cols, sorted, row_nnz, err;
  DevBuf<double> vals;
  keys.alloc(total);
  cols.alloc(total);
  sorted.alloc(total);
  if (data) vals.alloc(total);
  row_nnz.alloc(n_agg);
  err.alloc(1);
  MGPBD_CUDA(cudaMemsetAsync(keys.p, 0xff, sizeof(int32_t) * total, s));
  if (data) MGPBD_CUDA(cudaMemsetAsync(vals.p, 0, sizeof(double) * total, s));
  MGPBD_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int32_t), s));
  k_rap_rows<<<rb, 32 * kRapWarps, 0, s>>>(indptr, indices, data, agg, mem_ptr, mem_rows, n_agg,
                                           off.p, keys.p, data ? vals.p : nullptr, cols.p,
                                           sorted.p, row_nnz.p, err.p);
  MGPBD_CHECK_LAUNCH();
  int32_t herr = 0;
  MGPBD_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
  require(herr == 0, MGPBD_EINVAL, "device Galerkin: a row's hash table overflowed");
  // coarse row pointers
  std::vector<int32_t> h_nnz(n_agg);
  MGPBD_CUDA(cudaMemcpyAsync(h_nnz.data(), row_nnz.p, sizeof(int32_t) * n_agg,
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
  out.host_indptr.assign(static_cast<size_t>(n_agg) + 1, 0);
  int64_t nnz_c = 0;
  for (int32_t I = 0; I < n_agg; ++I) {
    nnz_c += h_nnz[I];
    require(nnz_c < INT32_MAX, MGPBD_ERANGE, "coarse nnz exceeds int32");
    out.host_indptr[I + 1] = static_cast<int32_t>(nnz_c);
  }
  out.nnz = nnz_c;
  out.indptr.alloc(static_cast<int64_t>(n_agg) + 1);
  MGPBD_CUDA(cudaMemcpyAsync(out.indptr.p, out.host_indptr.data(), sizeof(int32_t) * (n_agg + 1),
                             cudaMemcpyHostToDevice, s));
  out.indices.alloc(nnz_c + kCsrPad);
  MGPBD_CUDA(cudaMemsetAsync(out.indices.p, 0, sizeof(int32_t) * (nnz_c + kCsrPad), s));
  out.diag_pos.alloc(n_agg);
  MGPBD_CUDA(cudaMemsetAsync(out.diag_pos.p, 0xff, sizeof(int32_t) * n_agg, s));
  DevBuf<int32_t> cnt;
  cnt.alloc(nnz_c + 1);
  MGPBD_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (nnz_c + 1), s));
  k_rap_place<<<rb, 32 * kRapWarps, 0, s>>>(indptr, indices, agg, mem_ptr, mem_rows, n_agg,
                                            off.p, cols.p, out.indptr.p, out.indices.p,
                                            out.diag_pos.p, cnt.p);
  MGPBD_CHECK_LAUNCH();
  // contribution offsets (exclusive scan of the counts) and the map
  out.contrib_off.alloc(nnz_c + 1);
  exclusive_scan(cnt.p, nnz_c, out.contrib_off.p, s);
  int32_t nmap = 0;
  MGPBD_CUDA(cudaMemcpyAsync(&nmap, out.contrib_off.p + nnz_c, sizeof(int32_t),
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
  out.contrib_idx.alloc(std::max<int64_t>(nmap, 1));
  MGPBD_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (nnz_c + 1), s));
  k_rap_map<<<rb, 32 * kRapWarps, 0, s>>>(indptr, indices, agg, mem_ptr, mem_rows, n_agg,
                                          out.indptr.p, out.indices.p, out.contrib_off.p, cnt.p,
                                          out.contrib_idx.p);
  MGPBD_CHECK_LAUNCH();
  out.host_indices.resize(nnz_c);
  MGPBD_CUDA(cudaMemcpyAsync(out.host_indices.data(), out.indices.p, sizeof(int32_t) * nnz_c,
                             cudaMemcpyDeviceToHost, s));
  MGPBD_CUDA(cudaStreamSynchronize(s));
}

}  // namespace mgpbd
