// surrogate.cu - the learned surrogate's kernels on sm_103a: BF16 tensor-core convolutions
// (tcgen05.mma with FP32 accumulators in tensor memory, operands staged by TMA) for the
// forward pass, the data gradient and the weight gradient of a 1D convolution over
// channels-last activations, and the memory-bound steps around them (pooling, upsampling with
// skip concatenation, bias gradients, loss, Adam, input assembly, the training targets of a
// simulated band and per-map scores).  C ABI in include/mgpu_surrogate.h.
//
// A 1D convolution with `taps` taps (centre tap at offset `pad`) over X[B][L][Cin] is an
// implicit GEMM:
//   Y[b, l, n] = sum_t sum_c X[b, l + t - pad, c] * W[n][t][c]      (M = positions, N = Cout,
//                                                                    K = taps x Cin)
// TMA loads the A tile of tap t directly from X at row offset t - pad: rows outside [0, L)
// come back as zeros, which is the convolution's zero padding.  The data gradient is the same
// product with the taps reversed and W transposed; the weight gradient contracts over the
// positions (K = B x L) with both operands M/N-major.
//
// The forward kernels come in four forms (one CTA per tile or persistent; per-thread output
// rows or a staged epilogue that writes 32-row boxes to shared memory and stores them with
// TMA).  The staged epilogue can store the same box to several places at once, which lets a
// U-Net's convolutions fill their skip concatenations, upsampled halves and pooled inputs
// directly (msur_conv_forward_fused).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/mgpu_surrogate.h"
#include "umma.cuh"

namespace sg {

using bf16 = __nv_bfloat16;
constexpr int BM = 128;  // positions (or output channels in the weight gradient) per tile
constexpr int BK = 64;   // K elements per pipeline stage: one 128-byte swizzle row of BF16
constexpr int THREADS = 192;  // warp 0 TMA, warp 1 MMA (and TMEM), warps 2-5 epilogue

// Error bits of the kernels' bounded waits (msur_take_error).
enum : unsigned { ERR_PRODUCER = 1u, ERR_MMA = 2u, ERR_EPILOGUE = 4u };

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}
// SiLU and its derivative with the fast reciprocal-based division (within 2 ulp; the result is
// 0 when 1 + exp(-z) overflows, the limit of both): the epilogues evaluate one per output element.
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// ---------------------------------------------------------------------------------------
// Forward / data-gradient convolution: K-major A (activations) and B (weights)
// ---------------------------------------------------------------------------------------
struct ConvArgs {
  CUtensorMap tm_a;  // activations [B][L][Cin]: dims {Cin, L, B}, box {64, 128, 1}
  CUtensorMap tm_b;  // weights [N][taps * Cin]: dims {taps * Cin, N}, box {64, BN}
  int B, L, Cin, taps, pad;
  int n_valid;     // output channels written (columns >= n_valid are dropped)
  int out_stride;  // elements per output row
  int act;         // MSUR_ACT_*
  const float* bias;   // [n_valid] or null
  const bf16* gate;    // multiply by silu'(gate[row, col]) (row stride out_stride) or null
  bf16* out_pre;       // value before the activation, or null
  bf16* out_post;      // value after the activation, or null
  float* out_f32;      // FP32 value before the activation, or null
  unsigned* err;
  // staged epilogue (no gate): each epilogue warp writes its 32 rows of a 64-column unit to
  // shared memory and stores them with TMA.  Maps over [B][L][n_valid] with row stride
  // out_stride and 128-byte swizzled boxes of 32 rows: FP32 boxes of 32 columns, BF16 of 64.
  CUtensorMap tm_f32, tm_pre, tm_post;
  // fused copies of the post-activation output (staged epilogue only): a second copy into
  // another row-strided buffer (the skip half of a concatenation), and an upsampled copy, each
  // output row l stored at rows 2l and 2l + 1 of its buffer (two maps over the even and the odd
  // rows); out_post may then be null
  CUtensorMap tm_skip, tm_dup0, tm_dup1;
  // and an average-pooled copy: rows 2m and 2m + 1 (lanes 2m, 2m + 1 of an epilogue warp) into
  // row m, as msur_pool2 computes it from the BF16 values (16-row boxes)
  CUtensorMap tm_pool;
  int has_skip, has_dup, has_pool;
};

constexpr int STAGE_OUT_BYTES = 4 * 2 * 4096;  // four epilogue warps x two 4 KB buffers

template <int BN>
__host__ __device__ constexpr uint32_t tmem_cols() {
  return BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : (BN <= 256 ? 256 : 512)));
}

// Epilogue of one 32-column chunk of one output row: bias, the gated SiLU derivative, and
// the FP32 / pre-activation / post-activation stores (columns >= n_valid dropped).
__device__ __forceinline__ void conv_epilogue_chunk(const ConvArgs& a, float (&v)[32], size_t row, int col0) {
  const int nv = min(32, a.n_valid - col0);
  const size_t off = row * a.out_stride + col0;
  if (a.bias) {
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] += (j < nv) ? __ldg(a.bias + col0 + j) : 0.0f;
  }
  if (a.gate) {
    if (nv == 32) {
      const uint4* g4 = reinterpret_cast<const uint4*>(a.gate + off);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint4 u = __ldg(g4 + k);
        const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const __nv_bfloat162 g2 = *reinterpret_cast<const __nv_bfloat162*>(&w4[h]);
          v[8 * k + 2 * h] *= dsilu(__low2float(g2));
          v[8 * k + 2 * h + 1] *= dsilu(__high2float(g2));
        }
      }
    } else {
      for (int j = 0; j < nv; ++j) v[j] *= dsilu(__bfloat162float(a.gate[off + j]));
    }
  }
  if (a.out_f32) {
    if (nv == 32) {
      float4* o4 = reinterpret_cast<float4*>(a.out_f32 + off);
#pragma unroll
      for (int k = 0; k < 8; ++k) o4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else {
      for (int j = 0; j < nv; ++j) a.out_f32[off + j] = v[j];
    }
  }
  if (a.out_pre) {
    if (nv == 32) {
      uint4* o4 = reinterpret_cast<uint4*>(a.out_pre + off);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        uint32_t w4[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const __nv_bfloat162 p = __floats2bfloat162_rn(v[8 * k + 2 * h], v[8 * k + 2 * h + 1]);
          w4[h] = *reinterpret_cast<const uint32_t*>(&p);
        }
        o4[k] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
      }
    } else {
      for (int j = 0; j < nv; ++j) a.out_pre[off + j] = __float2bfloat16(v[j]);
    }
  }
  if (a.out_post) {
    if (a.act == MSUR_ACT_SILU) {
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] = silu(v[j]);
    }
    if (nv == 32) {
      uint4* o4 = reinterpret_cast<uint4*>(a.out_post + off);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        uint32_t w4[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const __nv_bfloat162 p = __floats2bfloat162_rn(v[8 * k + 2 * h], v[8 * k + 2 * h + 1]);
          w4[h] = *reinterpret_cast<const uint32_t*>(&p);
        }
        o4[k] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
      }
    } else {
      for (int j = 0; j < nv; ++j) a.out_post[off + j] = __float2bfloat16(v[j]);
    }
  }
}

// One 32-row x 128-byte box goes through this warp's staging buffer (two 4 KB buffers used in
// turn; nb counts the warp's stores).  stage_begin waits until the buffer's previous store has
// read it; the lanes then write their rows with the 128-byte swizzle (16-byte unit k of row r at
// unit k ^ (r % 8), which also keeps the eight lanes of each vector store on distinct banks);
// stage_end makes the writes visible to the bulk-copy proxy and lane 0 issues the TMA store.
__device__ __forceinline__ uint8_t* stage_begin(uint8_t* stg, int nb) {
  if (nb >= 2 && (threadIdx.x & 31) == 0) umma::bulk_wait_read<1>();
  __syncwarp();
  return stg + (nb & 1) * 4096;
}
__device__ __forceinline__ void stage_put(uint8_t* buf, int k, uint4 w) {
  const int lane = threadIdx.x & 31;
  *reinterpret_cast<uint4*>(buf + lane * 128 + ((k ^ (lane & 7)) << 4)) = w;
}
__device__ __forceinline__ void stage_end(const CUtensorMap* map, uint8_t* buf, int& nb, int x, int y, int z) {
  umma::fence_async_smem();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    umma::tma_store_3d(map, buf, x, y, z);
    umma::bulk_commit();
  }
  ++nb;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&p);
}

// Staged epilogue of one tile row block (32 rows y .. y+31 of sequence z, columns n0 .. n0+BN):
// per 64-column unit, bias, then the FP32 (two boxes), pre-activation and post-activation (one
// box each) outputs through shared memory and TMA.  Rows >= L and columns >= n_valid are dropped
// by the stores.  Collective over the warp; the caller waits for the stores (bulk_wait_all)
// before the block exits.
template <int BN>
__device__ void conv_epilogue_staged(const ConvArgs& a, uint32_t tmem_row, uint8_t* stg, int& nb, int n0, int y,
                                     int z) {
#pragma unroll 1
  for (int u = 0; u < BN / 64; ++u) {
    float v[64];
    umma::tmem_ld32(tmem_row + u * 64, *reinterpret_cast<float(*)[32]>(v));
    umma::tmem_ld32(tmem_row + u * 64 + 32, *reinterpret_cast<float(*)[32]>(v + 32));
    const int col0 = n0 + u * 64;
    if (y >= a.L || col0 >= a.n_valid) continue;
    if (a.bias) {
      const int nv = min(64, a.n_valid - col0);
      if (nv == 64 && (reinterpret_cast<uintptr_t>(a.bias) & 15u) == 0) {
        const float4* b4 = reinterpret_cast<const float4*>(a.bias + col0);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const float4 bb = __ldg(b4 + k);
          v[4 * k] += bb.x;
          v[4 * k + 1] += bb.y;
          v[4 * k + 2] += bb.z;
          v[4 * k + 3] += bb.w;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 64; ++j) v[j] += (j < nv) ? __ldg(a.bias + col0 + j) : 0.0f;
      }
    }
    if (a.out_f32) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (col0 + 32 * h >= a.n_valid) break;
        uint8_t* buf = stage_begin(stg, nb);
#pragma unroll
        for (int k = 0; k < 8; ++k)
          stage_put(buf, k,
                    make_uint4(__float_as_uint(v[32 * h + 4 * k]), __float_as_uint(v[32 * h + 4 * k + 1]),
                               __float_as_uint(v[32 * h + 4 * k + 2]), __float_as_uint(v[32 * h + 4 * k + 3])));
        stage_end(&a.tm_f32, buf, nb, col0 + 32 * h, y, z);
      }
    }
    if (a.out_pre) {
      uint8_t* buf = stage_begin(stg, nb);
#pragma unroll
      for (int k = 0; k < 8; ++k)
        stage_put(buf, k,
                  make_uint4(pack_bf16x2(v[8 * k], v[8 * k + 1]), pack_bf16x2(v[8 * k + 2], v[8 * k + 3]),
                             pack_bf16x2(v[8 * k + 4], v[8 * k + 5]), pack_bf16x2(v[8 * k + 6], v[8 * k + 7])));
      stage_end(&a.tm_pre, buf, nb, col0, y, z);
    }
    if (a.out_post || a.has_skip || a.has_dup || a.has_pool) {
      if (a.act == MSUR_ACT_SILU) {
#pragma unroll
        for (int j = 0; j < 64; ++j) v[j] = silu(v[j]);
      }
      uint32_t pk[32];  // this row's 64 BF16 values in pairs
#pragma unroll
      for (int j = 0; j < 32; ++j) pk[j] = pack_bf16x2(v[2 * j], v[2 * j + 1]);
      if (a.out_post || a.has_skip || a.has_dup) {
        uint8_t* buf = stage_begin(stg, nb);
#pragma unroll
        for (int k = 0; k < 8; ++k) stage_put(buf, k, make_uint4(pk[4 * k], pk[4 * k + 1], pk[4 * k + 2], pk[4 * k + 3]));
        // one staged box, stored to every destination of the post-activation value
        umma::fence_async_smem();
        __syncwarp();
        if ((threadIdx.x & 31) == 0) {
          if (a.out_post) umma::tma_store_3d(&a.tm_post, buf, col0, y, z);
          if (a.has_skip) umma::tma_store_3d(&a.tm_skip, buf, col0, y, z);
          if (a.has_dup) {
            umma::tma_store_3d(&a.tm_dup0, buf, col0, y, z);
            umma::tma_store_3d(&a.tm_dup1, buf, col0, y, z);
          }
          umma::bulk_commit();
        }
        ++nb;
      }
      if (a.has_pool) {
        // row pairs (2m, 2m + 1) sit on lanes (2m, 2m + 1): the even lane averages them and
        // writes pooled row m of a 16-row box (y is a multiple of 32)
        const int lane = threadIdx.x & 31;
        uint8_t* buf = stage_begin(stg, nb);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          uint32_t q[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const uint32_t mine = pk[4 * k + h];
            const uint32_t next = __shfl_down_sync(0xFFFFFFFFu, mine, 1);
            const float2 fa = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&mine));
            const float2 fb = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&next));
            q[h] = pack_bf16x2(0.5f * (fa.x + fb.x), 0.5f * (fa.y + fb.y));
          }
          if ((lane & 1) == 0) {
            const int r = lane >> 1;
            *reinterpret_cast<uint4*>(buf + r * 128 + ((k ^ (r & 7)) << 4)) = make_uint4(q[0], q[1], q[2], q[3]);
          }
        }
        stage_end(&a.tm_pool, buf, nb, col0, y >> 1, z);
      }
    }
  }
}

// Every TMA store of this warp has completed (before the block and its shared memory exit).
__device__ __forceinline__ void staged_drain() {
  if ((threadIdx.x & 31) == 0) umma::bulk_wait_all();
  __syncwarp();
}

template <int BN, int STAGES, bool STAGED>
__global__ void __launch_bounds__(THREADS, 1) conv_fwd_kernel(const __grid_constant__ ConvArgs a) {
  constexpr int A_BYTES = BM * BK * 2;
  constexpr int B_BYTES = BN * BK * 2;
  constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr uint32_t TCOLS = tmem_cols<BN>();
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int n0 = blockIdx.x * BN, l0 = blockIdx.y * BM, b = blockIdx.z;
  const int kc = a.Cin / BK;
  const int nk = a.taps * kc;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    umma::mbar_init(done, 1);
    umma::fence_barrier_init();
    umma::tma_prefetch(&a.tm_a);
    umma::tma_prefetch(&a.tm_b);
  }
  if (warp == 1) umma::tmem_alloc(tmem_slot, TCOLS);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int s = 0; s < nk; ++s) {
        const int st = s % STAGES;
        const uint32_t ph = (s / STAGES) & 1;
        if (!umma::mbar_wait(&empty[st], ph ^ 1, a.err, ERR_PRODUCER)) break;
        uint8_t* sa = smem + st * STAGE_BYTES;
        umma::mbar_arrive_expect_tx(&full[st], STAGE_BYTES);
        const int t = s / kc, c0 = (s % kc) * BK;
        umma::tma_load_3d(sa, &a.tm_a, &full[st], c0, l0 + t - a.pad, b);
        umma::tma_load_2d(sa + A_BYTES, &a.tm_b, &full[st], t * a.Cin + c0, n0);
        issued = s + 1;
      }
      // drain: every issued copy has landed before the block can exit
      for (int s = issued > STAGES ? issued - STAGES : 0; s < issued; ++s)
        umma::mbar_wait(&full[s % STAGES], (s / STAGES) & 1, a.err, ERR_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = umma::idesc_bf16_f32(BM, BN, false, false);
      for (int s = 0; s < nk; ++s) {
        const int st = s % STAGES;
        const uint32_t ph = (s / STAGES) & 1;
        if (!umma::mbar_wait(&full[st], ph, a.err, ERR_MMA)) break;
        umma::fence_after_sync();
        const uint32_t sa = umma::smem_u32(smem + st * STAGE_BYTES);
        const uint32_t sb = sa + A_BYTES;
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          umma::mma_bf16(tmem, umma::sdesc_sw128(sa + kk * 32, 16, 1024), umma::sdesc_sw128(sb + kk * 32, 16, 1024),
                         idesc, (s | kk) != 0);
        }
        umma::mma_commit(&empty[st]);
      }
      umma::mma_commit(done);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, one output row per thread
    const int q = warp & 3;
    const int l = l0 + 32 * q + lane;
    const bool row_ok = l < a.L;
    const size_t row = static_cast<size_t>(b) * a.L + (row_ok ? l : 0);
    const bool ok = umma::mbar_wait(done, 0, a.err, ERR_EPILOGUE);
    umma::fence_after_sync();
    if constexpr (STAGED) {
      if (ok) {
        int nb = 0;
        conv_epilogue_staged<BN>(a, tmem + (static_cast<uint32_t>(32 * q) << 16),
                                 smem + STAGES * STAGE_BYTES + 1024 + q * 8192, nb, n0, l0 + 32 * q, b);
        staged_drain();
      }
    } else if (ok) {
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        float v[32];
        umma::tmem_ld32(tmem + (static_cast<uint32_t>(32 * q) << 16) + c * 32, v);
        const int col0 = n0 + c * 32;
        if (!row_ok || col0 >= a.n_valid) continue;
        conv_epilogue_chunk(a, v, row, col0);
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, TCOLS);
  }
}

// ---------------------------------------------------------------------------------------
// The same convolution as a persistent kernel: each CTA walks tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ... (N tile fastest, then position tile, then sequence) with a
// double-buffered TMEM accumulator, so the epilogue of one tile overlaps the MMAs of the next
// and a CTA's set-up (barriers, TMEM allocation, tensor-map prefetch) is paid once.
// Barriers: full / empty per smem stage (TMA <-> MMA), tfull / tempty per accumulator
// (MMA <-> the 128 epilogue threads), done (the MMA issuer's last commit).
// ---------------------------------------------------------------------------------------
template <int BN, int STAGES, bool STAGED>
__global__ void __launch_bounds__(THREADS, 1) conv_fwd_persistent_kernel(const __grid_constant__ ConvArgs a, int ntn,
                                                                         int ntl, int ntiles) {
  constexpr int A_BYTES = BM * BK * 2;
  constexpr int B_BYTES = BN * BK * 2;
  constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr uint32_t TCOLS = tmem_cols<2 * BN>();
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* done = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int kc = a.Cin / BK;
  const int nk = a.taps * kc;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    for (int k = 0; k < 2; ++k) {
      umma::mbar_init(&tfull[k], 1);
      umma::mbar_init(&tempty[k], 128);
    }
    umma::mbar_init(done, 1);
    umma::fence_barrier_init();
    umma::tma_prefetch(&a.tm_a);
    umma::tma_prefetch(&a.tm_b);
  }
  if (warp == 1) umma::tmem_alloc(tmem_slot, TCOLS);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int s = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int n0 = (t % ntn) * BN;
        const int l0 = ((t / ntn) % ntl) * BM;
        const int b = t / (ntn * ntl);
        for (int kk = 0; kk < nk; ++kk, ++s) {
          const int st = s % STAGES;
          if (!umma::mbar_wait(&empty[st], ((s / STAGES) & 1) ^ 1, a.err, ERR_PRODUCER)) {
            ok = false;
            break;
          }
          uint8_t* sa = smem + st * STAGE_BYTES;
          umma::mbar_arrive_expect_tx(&full[st], STAGE_BYTES);
          const int tap = kk / kc, c0 = (kk % kc) * BK;
          umma::tma_load_3d(sa, &a.tm_a, &full[st], c0, l0 + tap - a.pad, b);
          umma::tma_load_2d(sa + A_BYTES, &a.tm_b, &full[st], tap * a.Cin + c0, n0);
        }
      }
      // drain: every issued copy has landed before the block can exit
      for (int q = s > STAGES ? s - STAGES : 0; q < s; ++q)
        umma::mbar_wait(&full[q % STAGES], (q / STAGES) & 1, a.err, ERR_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = umma::idesc_bf16_f32(BM, BN, false, false);
      int s = 0, j = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++j) {
        const int acc = j & 1;
        if (!umma::mbar_wait(&tempty[acc], ((j >> 1) & 1) ^ 1, a.err, ERR_MMA)) break;
        umma::fence_after_sync();
        const uint32_t d = tmem + acc * BN;
        for (int kk = 0; kk < nk; ++kk, ++s) {
          const int st = s % STAGES;
          if (!umma::mbar_wait(&full[st], (s / STAGES) & 1, a.err, ERR_MMA)) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          const uint32_t sa = umma::smem_u32(smem + st * STAGE_BYTES);
          const uint32_t sb = sa + A_BYTES;
#pragma unroll
          for (int k4 = 0; k4 < BK / 16; ++k4) {
            umma::mma_bf16(d, umma::sdesc_sw128(sa + k4 * 32, 16, 1024), umma::sdesc_sw128(sb + k4 * 32, 16, 1024),
                           idesc, (kk | k4) != 0);
          }
          umma::mma_commit(&empty[st]);
        }
        if (ok) umma::mma_commit(&tfull[acc]);
      }
      // every MMA this thread issued has completed before TMEM is released
      umma::mma_commit(done);
      umma::mbar_wait(done, 0, a.err, ERR_MMA);
    }
  } else {
    const int q = warp & 3;
    int j = 0, nb = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++j) {
      const int acc = j & 1;
      const bool ok = umma::mbar_wait(&tfull[acc], (j >> 1) & 1, a.err, ERR_EPILOGUE);
      umma::fence_after_sync();
      if (!ok) break;
      const int n0 = (t % ntn) * BN;
      const int y = ((t / ntn) % ntl) * BM + 32 * q;
      const int b = t / (ntn * ntl);
      if constexpr (STAGED) {
        conv_epilogue_staged<BN>(a, tmem + (static_cast<uint32_t>(32 * q) << 16) + acc * BN,
                                 smem + STAGES * STAGE_BYTES + 1024 + q * 8192, nb, n0, y, b);
      } else {
        const int l = y + lane;
        const bool row_ok = l < a.L;
        const size_t row = static_cast<size_t>(b) * a.L + (row_ok ? l : 0);
#pragma unroll 1
        for (int c = 0; c < BN / 32; ++c) {
          float v[32];
          umma::tmem_ld32(tmem + (static_cast<uint32_t>(32 * q) << 16) + acc * BN + c * 32, v);
          const int col0 = n0 + c * 32;
          if (!row_ok || col0 >= a.n_valid) continue;
          conv_epilogue_chunk(a, v, row, col0);
        }
      }
      umma::fence_before_sync();
      umma::mbar_arrive(&tempty[acc]);
    }
    if constexpr (STAGED) staged_drain();
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, TCOLS);
  }
}

// ---------------------------------------------------------------------------------------
// Weight gradient: dW[n][t][c] += sum_{b,l} dZ[b, l, n] X[b, l + t - pad, c], split over the
// (b, 64-position block) range; M = output channels (128 per tile), N = input channels (BN per
// tile), one TMEM accumulator of BN columns per tap; both operands M/N-major.
// ---------------------------------------------------------------------------------------
struct WgradArgs {
  CUtensorMap tm_dz;  // [B][L][Cout]: dims {Cout, L, B}, box {64, 64, 1}
  CUtensorMap tm_x;   // [B][L][Cin]: dims {Cin, L, B}, box {64, 64, 1}
  int B, L, Cin, Cout, taps, pad;
  int lblocks;        // 64-position blocks per sequence
  int total;          // B * lblocks
  int per_split;      // blocks per split
  float* dw;          // [Cout][taps][Cin], accumulated into
  unsigned* err;
};

template <int BN, int NT, int STAGES>
__global__ void __launch_bounds__(THREADS, 1) wgrad_kernel(const __grid_constant__ WgradArgs a) {
  constexpr int BOX = 64 * 64 * 2;  // one 64 x 64 BF16 box
  constexpr int A_BYTES = 2 * BOX;  // 128 output channels
  constexpr int B_TAP = (BN / 64) * BOX;
  constexpr int STAGE_BYTES = A_BYTES + NT * B_TAP;
  constexpr uint32_t TCOLS = NT * BN <= 128 ? 128 : (NT * BN <= 256 ? 256 : 512);
  static_assert(NT * BN <= 512, "accumulators exceed tensor memory");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int c0 = blockIdx.x * BN, n0 = blockIdx.y * BM;
  const int kb0 = blockIdx.z * a.per_split;
  const int kb1 = min(a.total, kb0 + a.per_split);
  const int nk = kb1 > kb0 ? kb1 - kb0 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    umma::mbar_init(done, 1);
    umma::fence_barrier_init();
    umma::tma_prefetch(&a.tm_dz);
    umma::tma_prefetch(&a.tm_x);
  }
  if (warp == 1) umma::tmem_alloc(tmem_slot, TCOLS);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int s = 0; s < nk; ++s) {
        const int st = s % STAGES;
        const uint32_t ph = (s / STAGES) & 1;
        if (!umma::mbar_wait(&empty[st], ph ^ 1, a.err, ERR_PRODUCER)) break;
        uint8_t* sa = smem + st * STAGE_BYTES;
        const int kb = kb0 + s;
        const int bb = kb / a.lblocks, l0 = (kb % a.lblocks) * 64;
        umma::mbar_arrive_expect_tx(&full[st], STAGE_BYTES);
        umma::tma_load_3d(sa, &a.tm_dz, &full[st], n0, l0, bb);
        umma::tma_load_3d(sa + BOX, &a.tm_dz, &full[st], n0 + 64, l0, bb);
#pragma unroll
        for (int t = 0; t < NT; ++t) {
#pragma unroll
          for (int j = 0; j < BN / 64; ++j)
            umma::tma_load_3d(sa + A_BYTES + t * B_TAP + j * BOX, &a.tm_x, &full[st], c0 + 64 * j, l0 + t - a.pad, bb);
        }
        issued = s + 1;
      }
      for (int s = issued > STAGES ? issued - STAGES : 0; s < issued; ++s)
        umma::mbar_wait(&full[s % STAGES], (s / STAGES) & 1, a.err, ERR_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = umma::idesc_bf16_f32(BM, BN, true, true);
      for (int s = 0; s < nk; ++s) {
        const int st = s % STAGES;
        const uint32_t ph = (s / STAGES) & 1;
        if (!umma::mbar_wait(&full[st], ph, a.err, ERR_MMA)) break;
        umma::fence_after_sync();
        const uint32_t sa = umma::smem_u32(smem + st * STAGE_BYTES);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t ad = umma::sdesc_sw128(sa + kk * 2048, BOX, 1024);
#pragma unroll
          for (int t = 0; t < NT; ++t) {
            const uint64_t bd = umma::sdesc_sw128(sa + A_BYTES + t * B_TAP + kk * 2048, BOX, 1024);
            umma::mma_bf16(tmem + t * BN, ad, bd, idesc, (s | kk) != 0);
          }
        }
        umma::mma_commit(&empty[st]);
      }
      umma::mma_commit(done);
    }
  } else if (nk > 0) {
    const int q = warp & 3;
    const int n = n0 + 32 * q + lane;
    const bool ok = umma::mbar_wait(done, 0, a.err, ERR_EPILOGUE);
    umma::fence_after_sync();
    if (ok) {
#pragma unroll 1
      for (int t = 0; t < NT; ++t) {
#pragma unroll 1
        for (int c = 0; c < BN / 32; ++c) {
          float v[32];
          umma::tmem_ld32(tmem + (static_cast<uint32_t>(32 * q) << 16) + t * BN + c * 32, v);
          const int cc = c0 + c * 32;
          if (n >= a.Cout || cc >= a.Cin) continue;
          float* dst = a.dw + (static_cast<size_t>(n) * a.taps + t) * a.Cin + cc;
          const int nv = min(32, a.Cin - cc);
          for (int j = 0; j < nv; ++j) atomicAdd(dst + j, v[j]);
        }
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, TCOLS);
  }
}

// ---------------------------------------------------------------------------------------
// Memory-bound steps (channels-last BF16 unless noted)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ float ldbf(const bf16* p) { return __bfloat162float(*p); }

// y[b, l, c] = (x[b, 2l, c] + x[b, 2l + 1, c]) / 2, l < Lout
__global__ void pool2_kernel(const bf16* x, int B, int Lout, int C, bf16* y) {
  const size_t n = static_cast<size_t>(B) * Lout * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const size_t bl = i / C;
    const int l = bl % Lout;
    const int b = bl / Lout;
    const size_t src = (static_cast<size_t>(b) * 2 * Lout + 2 * l) * C + c;
    y[i] = __float2bfloat16(0.5f * (ldbf(x + src) + ldbf(x + src + C)));
  }
}

// dz[b, l, c] = (dpool[b, l/2, c] / 2 + dcat[b, l, cat_off + c]) * silu'(z[b, l, c]) over l < L
// (dpool may be null when L is odd at its end, dcat may be null)
__global__ void skip_grad_kernel(const bf16* dpool, int Lp, const bf16* dcat, int cat_stride, int cat_off,
                                 const bf16* z, int B, int L, int C, bf16* dz) {
  const size_t n = static_cast<size_t>(B) * L * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const size_t bl = i / C;
    const int l = bl % L;
    const int b = bl / L;
    float g = 0.0f;
    if (dpool && l / 2 < Lp) g += 0.5f * ldbf(dpool + (static_cast<size_t>(b) * Lp + l / 2) * C + c);
    if (dcat) g += ldbf(dcat + bl * cat_stride + cat_off + c);
    dz[i] = __float2bfloat16(g * dsilu(ldbf(z + i)));
  }
}

// out[b, l, :] = [x[b, l/2, 0:C1], skip[b, l, 0:C2]]
__global__ void upcat_kernel(const bf16* x, const bf16* skip, int B, int L, int C1, int C2, bf16* out) {
  const int C = C1 + C2;
  const size_t n = static_cast<size_t>(B) * L * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const size_t bl = i / C;
    const int l = bl % L;
    const int b = bl / L;
    out[i] = c < C1 ? x[(static_cast<size_t>(b) * (L / 2) + l / 2) * C1 + c] : skip[bl * C2 + (c - C1)];
  }
}

// dz[b, l', c] = (dcat[b, 2l', c] + dcat[b, 2l' + 1, c]) * silu'(z[b, l', c]), c < C1
__global__ void upcat_bwd_kernel(const bf16* dcat, const bf16* z, int B, int Lh, int C1, int C, bf16* dz) {
  const size_t n = static_cast<size_t>(B) * Lh * C1;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C1;
    const size_t bl = i / C1;
    const int l = bl % Lh;
    const int b = bl / Lh;
    const size_t r = static_cast<size_t>(b) * 2 * Lh + 2 * l;
    const float g = ldbf(dcat + r * C + c) + ldbf(dcat + (r + 1) * C + c);
    dz[i] = __float2bfloat16(g * dsilu(ldbf(z + i)));
  }
}

// ---- the same steps eight channels (16 bytes) per thread, for channel counts, strides and
// offsets that are multiples of 8 and 16-byte aligned buffers (every shape of the network)
__device__ __forceinline__ void ld8(const bf16* p, float (&f)[8]) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[k]);
    f[2 * k] = __low2float(h);
    f[2 * k + 1] = __high2float(h);
  }
}
__device__ __forceinline__ void st8(bf16* p, const float (&f)[8]) {
  uint32_t w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
    w[k] = *reinterpret_cast<const uint32_t*>(&h);
  }
  *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void pool2_v8_kernel(const bf16* x, int B, int Lout, int C, bf16* y) {
  const int C8 = C / 8;
  const size_t n = static_cast<size_t>(B) * Lout * C8;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(i % C8) * 8;
    const size_t bl = i / C8;  // b * Lout + l
    const size_t src = 2 * bl * C + c;  // row 2l of sequence b: (b * 2 Lout + 2 l) * C
    float a[8], b[8];
    ld8(x + src, a);
    ld8(x + src + C, b);
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 0.5f * (a[k] + b[k]);
    st8(y + bl * C + c, a);
  }
}

__global__ void skip_grad_v8_kernel(const bf16* dpool, int Lp, const bf16* dcat, int cat_stride, int cat_off,
                                    const bf16* z, int B, int L, int C, bf16* dz) {
  const int C8 = C / 8;
  const size_t n = static_cast<size_t>(B) * L * C8;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(i % C8) * 8;
    const size_t bl = i / C8;
    const int l = bl % L;
    const int b = bl / L;
    float g[8] = {0, 0, 0, 0, 0, 0, 0, 0}, t[8];
    if (dpool && l / 2 < Lp) {
      ld8(dpool + (static_cast<size_t>(b) * Lp + l / 2) * C + c, t);
#pragma unroll
      for (int k = 0; k < 8; ++k) g[k] += 0.5f * t[k];
    }
    if (dcat) {
      ld8(dcat + bl * cat_stride + cat_off + c, t);
#pragma unroll
      for (int k = 0; k < 8; ++k) g[k] += t[k];
    }
    ld8(z + bl * C + c, t);
#pragma unroll
    for (int k = 0; k < 8; ++k) g[k] *= dsilu(t[k]);
    st8(dz + bl * C + c, g);
  }
}

__global__ void upcat_v8_kernel(const bf16* x, const bf16* skip, int B, int L, int C1, int C2, bf16* out) {
  const int C = C1 + C2, C8 = C / 8;
  const size_t n = static_cast<size_t>(B) * L * C8;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(i % C8) * 8;
    const size_t bl = i / C8;
    const int l = bl % L;
    const int b = bl / L;
    const bf16* src = c < C1 ? x + (static_cast<size_t>(b) * (L / 2) + l / 2) * C1 + c : skip + bl * C2 + (c - C1);
    *reinterpret_cast<uint4*>(out + bl * C + c) = *reinterpret_cast<const uint4*>(src);
  }
}

__global__ void upcat_bwd_v8_kernel(const bf16* dcat, const bf16* z, int B, int Lh, int C1, int C, bf16* dz) {
  const int C8 = C1 / 8;
  const size_t n = static_cast<size_t>(B) * Lh * C8;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(i % C8) * 8;
    const size_t bl = i / C8;  // b * Lh + l
    const size_t r = 2 * bl;   // row 2l of sequence b in dcat
    float a[8], b[8], t[8];
    ld8(dcat + r * C + c, a);
    ld8(dcat + (r + 1) * C + c, b);
    ld8(z + bl * C1 + c, t);
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (a[k] + b[k]) * dsilu(t[k]);
    st8(dz + bl * C1 + c, a);
  }
}

// db[c] += sum over rows of dz[r * stride + c], c < C; one block column of 32 channels per block
__global__ void bias_grad_kernel(const bf16* dz, size_t rows, int C, int stride, float* db) {
  const int c = blockIdx.x * 32 + threadIdx.x;
  float s = 0.0f;
  if (c < C) {
    for (size_t r = blockIdx.y * (size_t)blockDim.y + threadIdx.y; r < rows; r += (size_t)gridDim.y * blockDim.y)
      s += ldbf(dz + r * stride + c);
  }
  __shared__ float red[8][33];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < C) {
    for (int k = 1; k < blockDim.y; ++k) s += red[k][threadIdx.x];
    atomicAdd(db + c, s);
  }
}

// Mean-squared error over n_valid channels of each row: loss += sum (p - t)^2 (FP64 per block),
// dp[r, c] = scale * (p - t) for c < n_valid and 0 for the padded channels up to dstride.
__global__ void mse_kernel(const float* pred, int pstride, const float* target, int tstride, size_t rows, int n_valid,
                           bf16* dp, int dstride, float scale, double* loss) {
  double acc = 0.0;
  const size_t n = rows * static_cast<size_t>(dstride);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % dstride;
    const size_t r = i / dstride;
    float g = 0.0f;
    if (c < n_valid) {
      const float d = pred[r * pstride + c] - target[r * tstride + c];
      acc += static_cast<double>(d) * d;
      g = scale * d;
    }
    if (dp) dp[i] = __float2bfloat16(g);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double red[32];
  if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += red[w];
    atomicAdd(loss, s);
  }
}

// Adam with decoupled weight decay on FP32 masters; also writes the BF16 copy the MMAs read.
__global__ void adam_kernel(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2,
                            float eps, float wd, float bc1, float bc2, float gscale, bf16* p_bf16) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i] * gscale;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float pi = p[i] * (1.0f - lr * wd);
    pi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    if (p_bf16) p_bf16[i] = __float2bfloat16(pi);
  }
}

// wt[c][t'][n] = w[n][taps - 1 - t'][c]: the data gradient's weights (transposed, taps reversed)
__global__ void weight_transpose_kernel(const bf16* w, int N, int taps, int C, bf16* wt) {
  const size_t n = static_cast<size_t>(N) * taps * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int o = i % N;
    const size_t ct = i / N;
    const int t = ct % taps;
    const int c = ct / taps;
    wt[i] = w[(static_cast<size_t>(o) * taps + (taps - 1 - t)) * C + c];
  }
}

// x[b, l, 0:4] = track[b][0:4][l], x[b, l, 4:8] = params[b][0:4], x[b, l, 8:C] = 0
__global__ void assemble_input_kernel(const float* track, const float* params, int B, int L, int C, bf16* x) {
  const size_t n = static_cast<size_t>(B) * L * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const size_t bl = i / C;
    const int l = bl % L;
    const int b = bl / L;
    float v = 0.0f;
    if (c < 4) v = track[(static_cast<size_t>(b) * 4 + c) * L + l];
    else if (c < 8) v = params[b * 4 + (c - 4)];
    x[i] = __float2bfloat16(v);
  }
}

// Training target of a summed band (column-major u32, ncols x nrows): per bin j (a column of
// the band, its nrows diagonals) T[j, d] = log1p(band[j, d] * nrows / sum_d band[j, d]), 0 for
// an empty bin.  One warp per bin.
__global__ void band_target_kernel(const uint32_t* band, size_t ncols, int nrows, float* out) {
  const size_t warps = (static_cast<size_t>(gridDim.x) * blockDim.x) / 32;
  for (size_t j = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) / 32; j < ncols; j += warps) {
    const uint32_t* col = band + j * nrows;
    unsigned long long s = 0;
    for (int d = threadIdx.x % 32; d < nrows; d += 32) s += col[d];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const double scale = s ? static_cast<double>(nrows) / static_cast<double>(s) : 0.0;
    for (int d = threadIdx.x % 32; d < nrows; d += 32)
      out[j * nrows + d] = static_cast<float>(log1p(static_cast<double>(col[d]) * scale));
  }
}

// Per map m (n values each): sums for Pearson r and relative L2 of pred against ref, in FP64:
// out[m] = {sum p', sum r', sum p'^2, sum r'^2, sum p' r', sum (p - r)^2} with p' = p - mean_p,
// r' = r - mean_r when means (2 per map) are given, the raw values otherwise: the two passes of
// the reference's Pearson (mean, then covariances of the deviations).
__global__ void map_sums_kernel(const float* pred, size_t pstride_map, const float* ref, size_t rstride_map,
                                size_t n, const double* means, double* out) {
  const int m = blockIdx.y;
  const float* p = pred + m * pstride_map;
  const float* r = ref + m * rstride_map;
  const double mp = means ? means[2 * m] : 0.0, mr = means ? means[2 * m + 1] : 0.0;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double a = p[i] - mp, b = r[i] - mr;
    s[0] += a;
    s[1] += b;
    s[2] += a * a;
    s[3] += b * b;
    s[4] += a * b;
    s[5] += (static_cast<double>(p[i]) - r[i]) * (static_cast<double>(p[i]) - r[i]);
  }
  __shared__ double red[6][32];
  for (int k = 0; k < 6; ++k) {
    double x = s[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (threadIdx.x % 32 == 0) red[k][threadIdx.x / 32] = x;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double x = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) x += red[threadIdx.x][w];
    atomicAdd(out + 6 * m + threadIdx.x, x);
  }
}

// Gather the first n_valid channels of rows with stride `stride` into a dense [rows][n_valid] FP32
// array (the head's padded output to the band layout), optionally in place-compatible.
__global__ void compact_rows_kernel(const float* in, int stride, size_t rows, int n_valid, float* out) {
  const size_t n = rows * static_cast<size_t>(n_valid);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = in[(i / n_valid) * stride + i % n_valid];
}

}  // namespace sg

// =========================================================================================
// Host side
// =========================================================================================
using namespace sg;

namespace {

thread_local char g_err[512];
std::mutex g_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
unsigned* g_dev_err[64] = {};
// pipeline stages of the forward/data-gradient convolution per N tile width (64, 128, 256):
// fewer stages let more CTAs share an SM, so one tile's epilogue overlaps another's main loop
int g_conv_stages[3] = {4, 3, 4};
// kernel form per N tile width: bit 0 the persistent kernel (double-buffered TMEM accumulator),
// bit 1 the staged epilogue (outputs through shared memory and TMA stores)
int g_conv_form[3] = {2, 2, 2};

int conv_slot(int bn) { return bn == 256 ? 2 : (bn == 128 ? 1 : 0); }

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return MSUR_OK;
  return fail(MSUR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int setup(unsigned** err) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return fail(MSUR_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  int dev = 0;
  int rc = cuda_ok(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= 64) return fail(MSUR_ERR_UNSUPPORTED, "device %d out of range", dev);
  if (!g_dev_err[dev]) {
    rc = cuda_ok(cudaMalloc(&g_dev_err[dev], sizeof(unsigned)), "cudaMalloc(error flag)");
    if (rc) return rc;
    rc = cuda_ok(cudaMemset(g_dev_err[dev], 0, sizeof(unsigned)), "cudaMemset(error flag)");
    if (rc) return rc;
  }
  *err = g_dev_err[dev];
  return MSUR_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// BF16 tensor map with 128-byte swizzling: dims[0] innermost.
int make_map(CUtensorMap* m, const void* base, int rank, const uint64_t* dims, const uint32_t* box) {
  cuuint64_t gd[3], gs[2];
  cuuint32_t bx[3], es[3] = {1, 1, 1};
  uint64_t stride = 2;
  for (int i = 0; i < rank; ++i) {
    gd[i] = dims[i];
    bx[i] = box[i];
    if (i > 0) gs[i - 1] = stride;
    stride *= dims[i];
  }
  const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, const_cast<void*>(base), gd, gs, bx, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MSUR_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", static_cast<int>(r));
  return MSUR_OK;
}

// Output map of the staged epilogue: [B][L][n_valid] elements of elem_bytes with row stride
// out_stride, boxes of box_x columns x 32 rows, 128-byte swizzle.
int make_out_map(CUtensorMap* m, void* base, CUtensorMapDataType type, int elem_bytes, int n_valid, int out_stride,
                 int L, int B, int box_x, int box_rows = 32) {
  const cuuint64_t gd[3] = {static_cast<cuuint64_t>(n_valid), static_cast<cuuint64_t>(L), static_cast<cuuint64_t>(B)};
  const cuuint64_t gs[2] = {static_cast<cuuint64_t>(out_stride) * elem_bytes,
                            static_cast<cuuint64_t>(out_stride) * elem_bytes * L};
  const cuuint32_t bx[3] = {static_cast<cuuint32_t>(box_x), static_cast<cuuint32_t>(box_rows), 1}, es[3] = {1, 1, 1};
  const CUresult r = g_encode(m, type, 3, base, gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MSUR_ERR_CUDA, "cuTensorMapEncodeTiled (output) failed (%d)", static_cast<int>(r));
  return MSUR_OK;
}

// Map of the upsampled copy: output row l of sequence b at element ((b * 2L + 2l + parity) *
// row_stride) of base, n_valid columns, boxes of 64 BF16 columns x 32 rows.
int make_dup_map(CUtensorMap* m, void* base, int parity, int n_valid, int row_stride, int L, int B) {
  const cuuint64_t gd[3] = {static_cast<cuuint64_t>(n_valid), static_cast<cuuint64_t>(L), static_cast<cuuint64_t>(B)};
  const cuuint64_t gs[2] = {static_cast<cuuint64_t>(row_stride) * 2 * 2,
                            static_cast<cuuint64_t>(row_stride) * 2 * 2 * L};
  const cuuint32_t bx[3] = {64, 32, 1}, es[3] = {1, 1, 1};
  void* b0 = static_cast<char*>(base) + static_cast<size_t>(parity) * row_stride * 2;
  const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, b0, gd, gs, bx, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MSUR_ERR_CUDA, "cuTensorMapEncodeTiled (upsampled) failed (%d)", static_cast<int>(r));
  return MSUR_OK;
}

// Dynamic shared memory of a forward kernel: operand stages, alignment slack, the barriers (a
// 1 KB block when the staged epilogue's buffers follow it).
template <int BN, int STAGES, bool STAGED>
constexpr int conv_smem() {
  return STAGES * (BM * BK * 2 + BN * BK * 2) + 1024 + (STAGED ? 1024 + STAGE_OUT_BYTES : 256);
}

template <int BN, int STAGES, bool STAGED>
int launch_conv(const ConvArgs& a, int ntiles_n, cudaStream_t st) {
  constexpr int smem = conv_smem<BN, STAGES, STAGED>();
  auto kern = conv_fwd_kernel<BN, STAGES, STAGED>;
  int rc = cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "smem attribute");
  if (rc) return rc;
  dim3 grid(ntiles_n, (a.L + BM - 1) / BM, a.B);
  kern<<<grid, THREADS, smem, st>>>(a);
  return cuda_ok(cudaGetLastError(), "conv_fwd_kernel launch");
}

template <int BN, int STAGES, bool STAGED>
int launch_conv_persistent(const ConvArgs& a, int ntn, cudaStream_t st) {
  constexpr int smem = conv_smem<BN, STAGES, STAGED>();
  constexpr int tcols = static_cast<int>(tmem_cols<2 * BN>());
  auto kern = conv_fwd_persistent_kernel<BN, STAGES, STAGED>;
  int rc = cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "smem attribute");
  if (rc) return rc;
  int dev = 0, sms = 0, per_sm = 0;
  rc = cuda_ok(cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc) rc = cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (!rc) rc = cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem), "occupancy");
  if (rc) return rc;
  per_sm = std::max(1, std::min(per_sm, 512 / tcols));  // each resident CTA holds its accumulators in TMEM
  const int ntl = (a.L + BM - 1) / BM;
  const int ntiles = ntn * ntl * a.B;
  const int grid = std::min(ntiles, sms * per_sm);
  kern<<<grid, THREADS, smem, st>>>(a, ntn, ntl, ntiles);
  return cuda_ok(cudaGetLastError(), "conv_fwd_persistent_kernel launch");
}

template <int BN, int STAGES>
int launch_conv_form(const ConvArgs& a, int ntn, bool persistent, bool staged, cudaStream_t st) {
  if (persistent) {
    return staged ? launch_conv_persistent<BN, STAGES, true>(a, ntn, st)
                  : launch_conv_persistent<BN, STAGES, false>(a, ntn, st);
  }
  return staged ? launch_conv<BN, STAGES, true>(a, ntn, st) : launch_conv<BN, STAGES, false>(a, ntn, st);
}

template <int BN>
int dispatch_conv(const ConvArgs& a, int ntn, bool persistent, bool staged, int stages, cudaStream_t st) {
  if (stages == 2) return launch_conv_form<BN, 2>(a, ntn, persistent, staged, st);
  if (stages == 3) return launch_conv_form<BN, 3>(a, ntn, persistent, staged, st);
  return launch_conv_form<BN, 4>(a, ntn, persistent, staged, st);
}

template <int BN, int NT, int STAGES>
int launch_wgrad(const WgradArgs& a, int splits, cudaStream_t st) {
  constexpr int smem = STAGES * (2 * 8192 + NT * (BN / 64) * 8192) + 1024 + 256;
  auto kern = wgrad_kernel<BN, NT, STAGES>;
  int rc = cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "smem attribute");
  if (rc) return rc;
  dim3 grid((a.Cin + BN - 1) / BN, (a.Cout + BM - 1) / BM, splits);
  kern<<<grid, THREADS, smem, st>>>(a);
  return cuda_ok(cudaGetLastError(), "wgrad_kernel launch");
}

unsigned grid_for(size_t n, unsigned block = 256) {
  const size_t g = (n + block - 1) / block;
  return static_cast<unsigned>(g < 152 * 32 ? (g ? g : 1) : 152 * 32);
}

}  // namespace

extern "C" {

const char* msur_last_error_string(void) { return g_err; }

int msur_take_error(unsigned* code) {
  unsigned* err = nullptr;
  int rc = setup(&err);
  if (rc) return rc;
  unsigned h = 0;
  rc = cuda_ok(cudaMemcpy(&h, err, sizeof(h), cudaMemcpyDeviceToHost), "read error flag");
  if (rc) return rc;
  if (h) rc = cuda_ok(cudaMemset(err, 0, sizeof(unsigned)), "clear error flag");
  if (code) *code = h;
  return rc;
}

static int conv_forward_impl(const void* x, int B, int L, int Cin, const void* w, int Cout, int taps,
                             const float* bias, int act, void* out_pre, void* out_post, float* out_f32,
                             int out_stride, int n_valid, const void* gate, void* out_skip, int skip_stride,
                             void* out_dup, int dup_stride, void* out_pool, int pool_stride, void* stream) {
  if (!x || !w || B <= 0 || L <= 0 || Cin <= 0 || Cout <= 0 || taps <= 0 || n_valid <= 0 || n_valid > Cout)
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward: bad shape or null pointer");
  if (Cin % BK) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward: Cin (%d) must be a multiple of 64", Cin);
  if (taps % 2 == 0) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward: taps must be odd");
  if (!out_pre && !out_post && !out_f32 && !out_skip && !out_dup && !out_pool)
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward: no output");
  if (out_pool && (L % 2)) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward_fused: pooling needs an even L");
  if ((out_skip && (skip_stride < n_valid || (skip_stride % 8) || !aligned16(out_skip))) ||
      (out_dup && (dup_stride < n_valid || (dup_stride % 8) || !aligned16(out_dup))) ||
      (out_pool && (pool_stride < n_valid || (pool_stride % 8) || !aligned16(out_pool))))
    return fail(MSUR_ERR_INVALID_ARG,
                "msur_conv_forward_fused: copies must be 16-byte aligned, their strides multiples of 8 and >= n_valid");
  const bool primary = out_pre || out_post || out_f32;
  if ((primary && (out_stride < n_valid || (out_stride % 8))) ||
      !aligned16(x) || !aligned16(w) || (out_pre && !aligned16(out_pre)) || (out_post && !aligned16(out_post)) ||
      (out_f32 && !aligned16(out_f32)) || (gate && !aligned16(gate)))
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward: buffers must be 16-byte aligned, out_stride a multiple of 8");
  if (act != MSUR_ACT_NONE && act != MSUR_ACT_SILU) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_forward: bad act");
  unsigned* err = nullptr;
  int rc = setup(&err);
  if (rc) return rc;
  const int BN = Cout <= 64 ? 64 : (Cout % 256 == 0 ? 256 : 128);
  ConvArgs a;
  std::memset(&a, 0, sizeof(a));
  const uint64_t dims_a[3] = {static_cast<uint64_t>(Cin), static_cast<uint64_t>(L), static_cast<uint64_t>(B)};
  const uint32_t box_a[3] = {64, BM, 1};
  rc = make_map(&a.tm_a, x, 3, dims_a, box_a);
  if (rc) return rc;
  const uint64_t dims_b[2] = {static_cast<uint64_t>(taps) * Cin, static_cast<uint64_t>(Cout)};
  const uint32_t box_b[2] = {64, static_cast<uint32_t>(BN)};
  rc = make_map(&a.tm_b, w, 2, dims_b, box_b);
  if (rc) return rc;
  a.B = B;
  a.L = L;
  a.Cin = Cin;
  a.taps = taps;
  a.pad = (taps - 1) / 2;
  a.n_valid = n_valid;
  a.out_stride = out_stride;
  a.act = act;
  a.bias = bias;
  a.gate = static_cast<const bf16*>(gate);
  a.out_pre = static_cast<bf16*>(out_pre);
  a.out_post = static_cast<bf16*>(out_post);
  a.out_f32 = out_f32;
  a.err = err;
  const int ntn = (Cout + BN - 1) / BN;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int slot = BN == 256 ? 2 : (BN == 128 ? 1 : 0);
  const int stages = g_conv_stages[slot];
  // kernel form: bit 0 the persistent kernel, bit 1 the staged epilogue (outputs through shared
  // memory and TMA), which needs no gate: the data gradient's gate is read row by row, so that
  // epilogue stays per thread
  const int form = g_conv_form[slot];
  const bool persistent = (form & 1) != 0;
  const bool staged = (form & 2) != 0 && !gate;
  if ((out_skip || out_dup || out_pool) && !staged)
    return fail(MSUR_ERR_UNSUPPORTED, "msur_conv_forward_fused: the fused copies need the staged form (bit 1) "
                                      "for N tile %d and no gate", BN);
  if (staged) {
    if (out_f32) rc = make_out_map(&a.tm_f32, out_f32, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, n_valid, out_stride, L, B, 32);
    if (!rc && out_pre)
      rc = make_out_map(&a.tm_pre, out_pre, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, n_valid, out_stride, L, B, 64);
    if (!rc && out_post)
      rc = make_out_map(&a.tm_post, out_post, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, n_valid, out_stride, L, B, 64);
    if (!rc && out_skip)
      rc = make_out_map(&a.tm_skip, out_skip, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, n_valid, skip_stride, L, B, 64);
    if (!rc && out_dup) rc = make_dup_map(&a.tm_dup0, out_dup, 0, n_valid, dup_stride, L, B);
    if (!rc && out_dup) rc = make_dup_map(&a.tm_dup1, out_dup, 1, n_valid, dup_stride, L, B);
    if (!rc && out_pool)
      rc = make_out_map(&a.tm_pool, out_pool, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, n_valid, pool_stride, L / 2, B, 64,
                        16);
    if (rc) return rc;
    a.has_skip = out_skip ? 1 : 0;
    a.has_dup = out_dup ? 1 : 0;
    a.has_pool = out_pool ? 1 : 0;
  }
  if (BN == 256) return dispatch_conv<256>(a, ntn, persistent, staged, stages, st);
  if (BN == 128) return dispatch_conv<128>(a, ntn, persistent, staged, stages, st);
  return dispatch_conv<64>(a, ntn, persistent, staged, stages, st);
}

int msur_conv_forward(const void* x, int B, int L, int Cin, const void* w, int Cout, int taps, const float* bias,
                      int act, void* out_pre, void* out_post, float* out_f32, int out_stride, int n_valid,
                      const void* gate, void* stream) {
  return conv_forward_impl(x, B, L, Cin, w, Cout, taps, bias, act, out_pre, out_post, out_f32, out_stride, n_valid,
                           gate, nullptr, 0, nullptr, 0, nullptr, 0, stream);
}

int msur_conv_forward_fused(const void* x, int B, int L, int Cin, const void* w, int Cout, int taps,
                            const float* bias, int act, void* out_post, int out_stride, void* out_skip,
                            int skip_stride, void* out_dup, int dup_stride, void* out_pool, int pool_stride,
                            int n_valid, void* stream) {
  return conv_forward_impl(x, B, L, Cin, w, Cout, taps, bias, act, nullptr, out_post, nullptr, out_stride, n_valid,
                           nullptr, out_skip, skip_stride, out_dup, dup_stride, out_pool, pool_stride, stream);
}

int msur_conv_set_stages(int bn, int stages) {
  if ((bn != 64 && bn != 128 && bn != 256) || stages < 2 || stages > 4)
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_set_stages: N tile 64, 128 or 256 and 2 to 4 stages");
  std::lock_guard<std::mutex> lk(g_mu);
  g_conv_stages[bn == 256 ? 2 : (bn == 128 ? 1 : 0)] = stages;
  return MSUR_OK;
}

int msur_conv_set_form(int bn, int form) {
  if ((bn != 64 && bn != 128 && bn != 256) || form < 0 || form > 3)
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_set_form: N tile 64, 128 or 256 and form 0 to 3");
  std::lock_guard<std::mutex> lk(g_mu);
  g_conv_form[conv_slot(bn)] = form;
  return MSUR_OK;
}

int msur_conv_get_form(int bn) {
  if (bn != 64 && bn != 128 && bn != 256) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_get_form: bad N tile");
  return g_conv_form[conv_slot(bn)];
}

int msur_conv_set_persistent(int bn, int on) {
  if (bn != 64 && bn != 128 && bn != 256) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_set_persistent: bad N tile");
  std::lock_guard<std::mutex> lk(g_mu);
  int& f = g_conv_form[conv_slot(bn)];
  f = (f & 2) | (on ? 1 : 0);
  return MSUR_OK;
}

int msur_conv_get_persistent(int bn) {
  if (bn != 64 && bn != 128 && bn != 256) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_get_persistent: bad N tile");
  return g_conv_form[conv_slot(bn)] & 1;
}

int msur_conv_get_stages(int bn) {
  if (bn != 64 && bn != 128 && bn != 256) return fail(MSUR_ERR_INVALID_ARG, "msur_conv_get_stages: bad N tile");
  return g_conv_stages[bn == 256 ? 2 : (bn == 128 ? 1 : 0)];
}

int msur_conv_wgrad(const void* x, const void* dz, int B, int L, int Cin, int Cout, int taps, float* dw, int splits,
                    void* stream) {
  if (!x || !dz || !dw || B <= 0 || L <= 0 || Cin <= 0 || Cout <= 0 || (taps != 1 && taps != 3))
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_wgrad: bad shape or null pointer (taps must be 1 or 3)");
  if ((Cin % 8) || (Cout % 8) || !aligned16(x) || !aligned16(dz))
    return fail(MSUR_ERR_INVALID_ARG, "msur_conv_wgrad: channels must be multiples of 8, buffers 16-byte aligned");
  unsigned* err = nullptr;
  int rc = setup(&err);
  if (rc) return rc;
  WgradArgs a;
  std::memset(&a, 0, sizeof(a));
  const uint64_t dz_dims[3] = {static_cast<uint64_t>(Cout), static_cast<uint64_t>(L), static_cast<uint64_t>(B)};
  const uint64_t x_dims[3] = {static_cast<uint64_t>(Cin), static_cast<uint64_t>(L), static_cast<uint64_t>(B)};
  const uint32_t box[3] = {64, 64, 1};
  rc = make_map(&a.tm_dz, dz, 3, dz_dims, box);
  if (!rc) rc = make_map(&a.tm_x, x, 3, x_dims, box);
  if (rc) return rc;
  a.B = B;
  a.L = L;
  a.Cin = Cin;
  a.Cout = Cout;
  a.taps = taps;
  a.pad = (taps - 1) / 2;
  a.lblocks = (L + 63) / 64;
  a.total = B * a.lblocks;
  if (splits <= 0) {
    // enough CTAs for the machine: about two waves of 152 SMs over the (n, c) tiles
    const int tiles = ((Cin + 127) / 128) * ((Cout + BM - 1) / BM);
    splits = (2 * 152 + tiles - 1) / tiles;
  }
  if (splits > a.total) splits = a.total;
  a.per_split = (a.total + splits - 1) / splits;
  splits = (a.total + a.per_split - 1) / a.per_split;
  a.dw = dw;
  a.err = err;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (taps == 3) {
    if (Cin <= 64) return launch_wgrad<64, 3, 4>(a, splits, st);
    return launch_wgrad<128, 3, 3>(a, splits, st);
  }
  return launch_wgrad<128, 1, 4>(a, splits, st);
}

int msur_pool2(const void* x, int B, int Lout, int C, void* y, void* stream) {
  if (!x || !y || B <= 0 || Lout <= 0 || C <= 0) return fail(MSUR_ERR_INVALID_ARG, "msur_pool2: bad argument");
  const size_t n = static_cast<size_t>(B) * Lout * C;
  if (C % 8 == 0 && aligned16(x) && aligned16(y)) {
    pool2_v8_kernel<<<grid_for(n / 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(x), B,
                                                                                   Lout, C, static_cast<bf16*>(y));
    return cuda_ok(cudaGetLastError(), "pool2_v8_kernel launch");
  }
  pool2_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(x), B, Lout, C,
                                                                           static_cast<bf16*>(y));
  return cuda_ok(cudaGetLastError(), "pool2_kernel launch");
}

int msur_skip_grad(const void* dpool, int Lp, const void* dcat, int cat_stride, int cat_off, const void* z, int B,
                   int L, int C, void* dz, void* stream) {
  if (!z || !dz || B <= 0 || L <= 0 || C <= 0) return fail(MSUR_ERR_INVALID_ARG, "msur_skip_grad: bad argument");
  const size_t n = static_cast<size_t>(B) * L * C;
  if (C % 8 == 0 && cat_stride % 8 == 0 && cat_off % 8 == 0 && aligned16(z) && aligned16(dz) &&
      (!dpool || aligned16(dpool)) && (!dcat || aligned16(dcat))) {
    skip_grad_v8_kernel<<<grid_for(n / 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(dpool), Lp, static_cast<const bf16*>(dcat), cat_stride, cat_off,
        static_cast<const bf16*>(z), B, L, C, static_cast<bf16*>(dz));
    return cuda_ok(cudaGetLastError(), "skip_grad_v8_kernel launch");
  }
  skip_grad_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(dpool), Lp, static_cast<const bf16*>(dcat), cat_stride, cat_off,
      static_cast<const bf16*>(z), B, L, C, static_cast<bf16*>(dz));
  return cuda_ok(cudaGetLastError(), "skip_grad_kernel launch");
}

int msur_upcat(const void* x, const void* skip, int B, int L, int C1, int C2, void* out, void* stream) {
  if (!x || !skip || !out || B <= 0 || L <= 0 || (L % 2)) return fail(MSUR_ERR_INVALID_ARG, "msur_upcat: bad argument");
  const size_t n = static_cast<size_t>(B) * L * (C1 + C2);
  if (C1 % 8 == 0 && C2 % 8 == 0 && aligned16(x) && aligned16(skip) && aligned16(out)) {
    upcat_v8_kernel<<<grid_for(n / 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(x), static_cast<const bf16*>(skip), B, L, C1, C2, static_cast<bf16*>(out));
    return cuda_ok(cudaGetLastError(), "upcat_v8_kernel launch");
  }
  upcat_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(x), static_cast<const bf16*>(skip), B, L, C1, C2, static_cast<bf16*>(out));
  return cuda_ok(cudaGetLastError(), "upcat_kernel launch");
}

int msur_upcat_bwd(const void* dcat, const void* z, int B, int Lh, int C1, int C, void* dz, void* stream) {
  if (!dcat || !z || !dz || B <= 0 || Lh <= 0 || C1 > C) return fail(MSUR_ERR_INVALID_ARG, "msur_upcat_bwd: bad argument");
  const size_t n = static_cast<size_t>(B) * Lh * C1;
  if (C1 % 8 == 0 && C % 8 == 0 && aligned16(dcat) && aligned16(z) && aligned16(dz)) {
    upcat_bwd_v8_kernel<<<grid_for(n / 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(dcat), static_cast<const bf16*>(z), B, Lh, C1, C, static_cast<bf16*>(dz));
    return cuda_ok(cudaGetLastError(), "upcat_bwd_v8_kernel launch");
  }
  upcat_bwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(dcat), static_cast<const bf16*>(z), B, Lh, C1, C, static_cast<bf16*>(dz));
  return cuda_ok(cudaGetLastError(), "upcat_bwd_kernel launch");
}

int msur_bias_grad(const void* dz, uint64_t rows, int C, int stride, float* db, void* stream) {
  if (!dz || !db || C <= 0 || stride < C) return fail(MSUR_ERR_INVALID_ARG, "msur_bias_grad: bad argument");
  dim3 block(32, 8);
  const uint64_t gy = (rows + 8 * 64 - 1) / (8 * 64);
  dim3 grid((C + 31) / 32, static_cast<unsigned>(gy < 512 ? (gy ? gy : 1) : 512));
  bias_grad_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(dz), rows, C,
                                                                          stride, db);
  return cuda_ok(cudaGetLastError(), "bias_grad_kernel launch");
}

int msur_mse(const float* pred, int pstride, const float* target, int tstride, uint64_t rows, int n_valid, void* dp,
             int dstride, float scale, double* loss, void* stream) {
  if (!pred || !target || !loss || n_valid <= 0 || pstride < n_valid || tstride < n_valid || dstride < n_valid)
    return fail(MSUR_ERR_INVALID_ARG, "msur_mse: bad argument");
  const size_t n = rows * static_cast<size_t>(dstride);
  mse_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(pred, pstride, target, tstride, rows, n_valid,
                                                                         static_cast<bf16*>(dp), dstride, scale, loss);
  return cuda_ok(cudaGetLastError(), "mse_kernel launch");
}

int msur_adam(float* p, const float* g, float* m, float* v, uint64_t n, float lr, float b1, float b2, float eps,
              float wd, int step, float gscale, void* p_bf16, void* stream) {
  if (!p || !g || !m || !v || step <= 0) return fail(MSUR_ERR_INVALID_ARG, "msur_adam: bad argument");
  const float bc1 = 1.0f - std::pow(b1, static_cast<float>(step));
  const float bc2 = 1.0f - std::pow(b2, static_cast<float>(step));
  adam_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(p, g, m, v, n, lr, b1, b2, eps, wd, bc1,
                                                                          bc2, gscale, static_cast<bf16*>(p_bf16));
  return cuda_ok(cudaGetLastError(), "adam_kernel launch");
}

int msur_weight_transpose(const void* w, int N, int taps, int C, void* wt, void* stream) {
  if (!w || !wt || N <= 0 || taps <= 0 || C <= 0) return fail(MSUR_ERR_INVALID_ARG, "msur_weight_transpose: bad argument");
  const size_t n = static_cast<size_t>(N) * taps * C;
  weight_transpose_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(w), N,
                                                                                      taps, C, static_cast<bf16*>(wt));
  return cuda_ok(cudaGetLastError(), "weight_transpose_kernel launch");
}

int msur_assemble_input(const float* track, const float* params, int B, int L, int C, void* x, void* stream) {
  if (!track || !params || !x || C < 8 || (C % 8)) return fail(MSUR_ERR_INVALID_ARG, "msur_assemble_input: bad argument");
  const size_t n = static_cast<size_t>(B) * L * C;
  assemble_input_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(track, params, B, L, C,
                                                                                   static_cast<bf16*>(x));
  return cuda_ok(cudaGetLastError(), "assemble_input_kernel launch");
}

int msur_band_target(const uint32_t* band, uint64_t ncols, int nrows, float* out, void* stream) {
  if (!band || !out || nrows <= 0) return fail(MSUR_ERR_INVALID_ARG, "msur_band_target: bad argument");
  band_target_kernel<<<grid_for(ncols * 32), 256, 0, static_cast<cudaStream_t>(stream)>>>(band, ncols, nrows, out);
  return cuda_ok(cudaGetLastError(), "band_target_kernel launch");
}

int msur_map_sums(const float* pred, uint64_t pstride_map, const float* ref, uint64_t rstride_map, uint64_t n,
                  int nmaps, const double* means, double* out, void* stream) {
  if (!pred || !ref || !out || nmaps <= 0 || nmaps > 65535) return fail(MSUR_ERR_INVALID_ARG, "msur_map_sums: bad argument");
  dim3 grid(static_cast<unsigned>(std::min<uint64_t>((n + 255) / 256, 64)), nmaps);
  map_sums_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(pred, pstride_map, ref, rstride_map, n,
                                                                        means, out);
  return cuda_ok(cudaGetLastError(), "map_sums_kernel launch");
}

int msur_compact_rows(const float* in, int stride, uint64_t rows, int n_valid, float* out, void* stream) {
  if (!in || !out || n_valid <= 0 || stride < n_valid) return fail(MSUR_ERR_INVALID_ARG, "msur_compact_rows: bad argument");
  const size_t n = rows * static_cast<size_t>(n_valid);
  compact_rows_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(in, stride, rows, n_valid, out);
  return cuda_ok(cudaGetLastError(), "compact_rows_kernel launch");
}

}  // extern "C"
