// mgpu_pixels.cu - pixel table of a chromosome's contact band (the data Cooler's writer emits).
//
// Cooler::write_or_append_cmatrix_to_file (src/libmodle_io/cooler_write_impl.hpp:275-316) walks
// bin1 i over the band's columns and bin2 j from i to min(i + nrows, ncols) - 1 and keeps the
// non-zero counts; the count of (i, j) is the band entry at column j, row j - i
// (contact_matrix_internal_impl.hpp:19-42), i.e. band[j * nrows + j - i].  Row i of the table is
// therefore the diagonal band[i * nrows + r * (nrows + 1)], r < nrows.
//
// Three HBM-bound passes: the non-zero count of every bin1 row (one warp per row), an exclusive
// scan of the counts into the bin1 index (one block), and the write of the pixels (one warp
// per row, each lane's slot from a ballot prefix).  Adjacent warps walk adjacent diagonals, so
// each 32-byte sector of the band is fetched from DRAM about once per pass and reused from L2.

#include <cuda_runtime.h>

#include <cstdio>

#include "mgpu_internal.h"

namespace mgpu {

namespace {

constexpr unsigned FULLM = 0xFFFFFFFFu;

__global__ void __launch_bounds__(256) band_row_counts_kernel(const u32* __restrict__ band, u64 nrows,
                                                             u64 ncols, u32* __restrict__ counts) {
  const u64 lane = threadIdx.x & 31u;
  const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
  for (u64 i = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < ncols; i += nwarps) {
    const u64 len = min(nrows, ncols - i);
    const u32* row = band + i * nrows;
    u32 cnt = 0;
    for (u64 r = lane; r < len; r += 32) cnt += __ldg(row + r * (nrows + 1)) != 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(FULLM, cnt, o);
    if (lane == 0) counts[i] = cnt;
  }
}

// offsets[i] = sum of counts[0..i), offsets[ncols] = total; one block of 1024 threads.
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(const u32* __restrict__ counts, u64 n,
                                                             u64* __restrict__ offsets) {
  __shared__ u64 warp_sums[32];
  __shared__ u64 carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const u32 lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (u64 base = 0; base < n; base += blockDim.x) {
    const u64 i = base + threadIdx.x;
    const u64 v = i < n ? counts[i] : 0;
    u64 x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const u64 y = __shfl_up_sync(FULLM, x, d);
      if ((int)lane >= d) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      u64 w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const u64 y = __shfl_up_sync(FULLM, w, d);
        if ((int)lane >= d) w += y;
      }
      warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    const u64 before = carry + (warp ? warp_sums[warp - 1] : 0);
    if (i < n) offsets[i] = before + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) offsets[n] = carry;
}

__global__ void __launch_bounds__(256) band_pixels_kernel(const u32* __restrict__ band, u64 nrows, u64 ncols,
                                                         u64 bin_offset, const u64* __restrict__ offsets,
                                                         int64_t* __restrict__ bin1, int64_t* __restrict__ bin2,
                                                         u32* __restrict__ count) {
  const u32 lane = threadIdx.x & 31u;
  const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
  for (u64 i = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < ncols; i += nwarps) {
    const u64 len = min(nrows, ncols - i);
    const u32* row = band + i * nrows;
    u64 k = offsets[i];
    for (u64 r0 = 0; r0 < len; r0 += 32) {
      const u64 r = r0 + lane;
      const u32 m = r < len ? __ldg(row + r * (nrows + 1)) : 0u;
      const unsigned nz = __ballot_sync(FULLM, m != 0u);
      if (m != 0u) {
        const u64 at = k + __popc(nz & ((1u << lane) - 1u));
        bin1[at] = (int64_t)(bin_offset + i);
        bin2[at] = (int64_t)(bin_offset + i + r);
        count[at] = m;
      }
      k += __popc(nz);
    }
  }
}

int grid_for(const void* fn, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return sms * per_sm;
}

int fail_cuda(cudaError_t e, const char* what, char* errbuf, int errlen) {
  if (e == cudaSuccess) return MGPU_OK;
  if (errbuf) snprintf(errbuf, errlen, "%s: %s", what, cudaGetErrorString(e));
  return MGPU_ERR_CUDA;
}

}  // namespace

int launch_band_counts(const u32* band, u64 nrows, u64 ncols, u32* counts, u64* offsets, void* stream,
                       char* errbuf, int errlen) {
  cudaStream_t st = (cudaStream_t)stream;
  if (ncols > 0) {
    const int grid = grid_for((const void*)band_row_counts_kernel, 256);
    band_row_counts_kernel<<<grid, 256, 0, st>>>(band, nrows, ncols, counts);
    int rc = fail_cuda(cudaGetLastError(), "band_row_counts_kernel launch", errbuf, errlen);
    if (rc) return rc;
  }
  exclusive_scan_kernel<<<1, 1024, 0, st>>>(counts, ncols, offsets);
  return fail_cuda(cudaGetLastError(), "exclusive_scan_kernel launch", errbuf, errlen);
}

int launch_band_pixels(const u32* band, u64 nrows, u64 ncols, u64 bin_offset, const u64* offsets,
                       int64_t* bin1, int64_t* bin2, u32* count, void* stream, char* errbuf, int errlen) {
  if (ncols == 0) return MGPU_OK;
  const int grid = grid_for((const void*)band_pixels_kernel, 256);
  band_pixels_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(band, nrows, ncols, bin_offset, offsets, bin1,
                                                             bin2, count);
  return fail_cuda(cudaGetLastError(), "band_pixels_kernel launch", errbuf, errlen);
}

}  // namespace mgpu
