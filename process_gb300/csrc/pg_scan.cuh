// Exclusive prefix sums over rows of u32 / u64 values (three-pass:
// block totals, scan of totals, block scan with carry-in).  Used for the
// per-context tile tables of the genome index, the per-edge mutation offsets
// and the per-bucket offsets of the locus sort.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pg_kernels.h"

namespace pg {

constexpr int SCAN_BLOCK = 1024;   // elements per block (256 threads x 4)

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T n = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += n;
  }
  return v;
}

// block-wide exclusive scan of 4 consecutive values per thread (256 threads);
// returns the block total.
template <typename T>
__device__ __forceinline__ T block_excl_scan4(T (&v)[4], T* smem /* >= 8 */) {
  T s0 = v[0], s1 = s0 + v[1], s2 = s1 + v[2], s3 = s2 + v[3];
  T incl = warp_incl_scan(s3);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 31) smem[warp] = incl;
  __syncthreads();
  T wbase = 0, total = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) { T x = smem[w]; if (w < warp) wbase += x; total += x; }
  __syncthreads();
  const T base = wbase + incl - s3;
  v[3] = base + s2; v[2] = base + s1; v[1] = base + s0; v[0] = base;
  return total;
}

template <typename T>
__global__ void k_scan_partials(const T* __restrict__ in, T* __restrict__ part, uint64_t n, int nblk) {
  __shared__ T sm[8];
  const int row = blockIdx.y;
  const uint64_t base = uint64_t(blockIdx.x) * SCAN_BLOCK + threadIdx.x * 4;
  const T* rin = in + uint64_t(row) * n;
  T v[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = (base + i < n) ? rin[base + i] : T(0);
  T tot = block_excl_scan4(v, sm);
  if (threadIdx.x == 0) part[uint64_t(row) * nblk + blockIdx.x] = tot;
}

// one block per row: exclusive scan of the block totals in place; writes row total
template <typename T>
__global__ void k_scan_totals(T* __restrict__ part, int nblk, T* __restrict__ row_total) {
  __shared__ T sm[8];
  __shared__ T carry;
  const int row = blockIdx.x;
  T* p = part + uint64_t(row) * nblk;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b = 0; b < nblk; b += SCAN_BLOCK) {
    T v[4];
    const int base = b + threadIdx.x * 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = (base + i < nblk) ? p[base + i] : T(0);
    T tot = block_excl_scan4(v, sm);
    const T c = carry;
#pragma unroll
    for (int i = 0; i < 4; ++i) if (base + i < nblk) p[base + i] = v[i] + c;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && row_total) row_total[row] = carry;
}

template <typename T>
__global__ void k_scan_apply(const T* __restrict__ in, T* __restrict__ out, const T* __restrict__ part,
                             uint64_t n, int nblk) {
  __shared__ T sm[8];
  const int row = blockIdx.y;
  const uint64_t base = uint64_t(blockIdx.x) * SCAN_BLOCK + threadIdx.x * 4;
  const T* rin = in + uint64_t(row) * n;
  T* rout = out + uint64_t(row) * n;
  T v[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = (base + i < n) ? rin[base + i] : T(0);
  block_excl_scan4(v, sm);
  const T c = part[uint64_t(row) * nblk + blockIdx.x];
#pragma unroll
  for (int i = 0; i < 4; ++i) if (base + i < n) rout[base + i] = v[i] + c;
}

// Exclusive scan of `rows` rows of n elements each (in may alias out).
// `part` needs rows * ceil(n/SCAN_BLOCK) elements; row_total (optional) rows.
template <typename T>
inline void scan_rows(const T* in, T* out, uint64_t n, int rows, T* part, T* row_total, cudaStream_t st) {
  const int nblk = int((n + SCAN_BLOCK - 1) / SCAN_BLOCK);
  if (n == 0) {
    if (row_total) cudaMemsetAsync(row_total, 0, sizeof(T) * rows, st);
    return;
  }
  dim3 g(nblk, rows);
  k_scan_partials<T><<<g, 256, 0, st>>>(in, part, n, nblk);
  k_scan_totals<T><<<rows, 256, 0, st>>>(part, nblk, row_total);
  k_scan_apply<T><<<g, 256, 0, st>>>(in, out, part, n, nblk);
  note_launch(3);
}

inline uint64_t scan_part_elems(uint64_t n, int rows) {
  return uint64_t(rows) * ((n + SCAN_BLOCK - 1) / SCAN_BLOCK) + 1;
}

}  // namespace pg
