/*
 * mgpu_surrogate.h - C ABI of the learned surrogate's GPU kernels (libmgpu_surrogate.so).
 *
 * No counterpart in the reference: MoDLE only simulates.  The surrogate is a 1D U-Net that maps
 * a window's barrier track and extrusion parameters to the expected banded contact map the
 * simulator converges to; these are its building blocks, each one hand-written for sm_103a.
 * The convolutions run on the tensor cores (tcgen05.mma, BF16 operands staged by TMA, FP32
 * accumulators in tensor memory); the rest are memory-bound kernels.
 *
 * Conventions:
 *   - every pointer is device memory of the current device; activations are channels-last
 *     BF16 arrays [B][L][C] (C contiguous), weights BF16 [Cout][taps][Cin] with FP32 masters;
 *   - every call enqueues work on `stream` (a cudaStream_t, NULL = legacy default) and
 *     returns an int status (MSUR_OK == 0); msur_last_error_string() describes the failure;
 *   - the tensor-core kernels bound every wait on a barrier; a wait that runs out (about a
 *     second) sets a flag that msur_take_error() reads and clears, instead of hanging.
 */
#ifndef MGPU_SURROGATE_H
#define MGPU_SURROGATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSUR_OK 0
#define MSUR_ERR_INVALID_ARG (-1)
#define MSUR_ERR_CUDA (-2)
#define MSUR_ERR_UNSUPPORTED (-5)

#define MSUR_ACT_NONE 0
#define MSUR_ACT_SILU 1

const char* msur_last_error_string(void);
/* Read and clear the device error flag of the current device (synchronises): 0 = no wait of a
 * tensor-core kernel ran out since the last call; else bits 1 (TMA producer), 2 (MMA issuer),
 * 4 (epilogue). */
int msur_take_error(unsigned* code);

/*
 * Convolution over positions, as an implicit GEMM on the tensor cores:
 *   v[b, l, n] = bias[n] + sum_{t < taps} sum_{c < Cin} x[b, l + t - (taps - 1) / 2, c] * w[n][t][c]
 * (positions outside [0, L) read as zero), for n < n_valid (<= Cout); then
 *   gate != NULL: v *= silu'(gate[b, l, n])            (a data gradient through a SiLU)
 *   out_f32 [b, l, n] = v                              (FP32, e.g. the output head)
 *   out_pre [b, l, n] = v                              (BF16, kept for the backward pass)
 *   out_post[b, l, n] = act(v)                         (BF16, act = MSUR_ACT_NONE or SILU)
 * Outputs have rows of out_stride elements (a multiple of 8).  Cin must be a multiple of 64,
 * taps odd, buffers 16-byte aligned.  The data gradient of a convolution is this call on dz
 * with w replaced by msur_weight_transpose(w).
 */
int msur_conv_forward(const void* x, int B, int L, int Cin, const void* w, int Cout, int taps, const float* bias,
                      int act, void* out_pre, void* out_post, float* out_f32, int out_stride, int n_valid,
                      const void* gate, void* stream);

/* msur_conv_forward with the post-activation value (act applied; no pre-activation, FP32 or
 * gate) written to up to four places at once, for a U-Net's skip connections:
 *   out_post [B][L][out_stride] as in msur_conv_forward (or NULL);
 *   out_skip [B][L][skip_stride]: a second copy, e.g. the skip half of a concatenation buffer
 *            (pointer at that half's first channel; or NULL);
 *   out_dup  [B][2L][dup_stride]: nearest upsampling by two, output row l at rows 2l and 2l + 1
 *            (pointer at the first channel of the upsampled half; or NULL);
 *   out_pool [B][L/2][pool_stride]: average pooling by two of the BF16 values, exactly as
 *            msur_pool2 computes it (L even; or NULL).
 * Together with out_skip and out_pool of the encoder convolution, out_dup of the convolution
 * below a decoder level fills that level's concatenation buffer without msur_upcat or
 * msur_pool2.  The copies are TMA stores of the staged epilogue: MSUR_ERR_UNSUPPORTED unless
 * the form of this N tile width has bit 1.  Buffers 16-byte aligned, strides multiples of 8
 * and at least n_valid. */
int msur_conv_forward_fused(const void* x, int B, int L, int Cin, const void* w, int Cout, int taps,
                            const float* bias, int act, void* out_post, int out_stride, void* out_skip,
                            int skip_stride, void* out_dup, int dup_stride, void* out_pool, int pool_stride,
                            int n_valid, void* stream);

/* Pipeline depth of msur_conv_forward for one N tile width (64, 128 or 256 output channels per
 * tile, chosen by Cout): 2 to 4 shared-memory stages.  Fewer stages let 2-4 CTAs share an SM,
 * so that one tile's epilogue overlaps another's main loop; the autotuner
 * (modlefork_gb300/autotune.py) picks the depths per device.  Defaults 4 (64), 3 (128), 4 (256).
 * msur_conv_get_stages returns the current depth (negative on a bad width). */
int msur_conv_set_stages(int bn, int stages);
int msur_conv_get_stages(int bn);
/* Kernel form of msur_conv_forward for one N tile width, two bits:
 *   bit 0: a persistent kernel (CTAs walk the tiles with a double-buffered TMEM accumulator, so
 *          a tile's epilogue overlaps the next tile's MMAs) instead of one CTA per output tile;
 *   bit 1: the staged epilogue: each epilogue warp writes 32 rows x 64 columns of output to
 *          shared memory and stores them with a TMA store, instead of one row per thread
 *          (calls with a gate always take the per-thread epilogue).
 * Results are identical in every form; the default is 2 and the autotuner picks per device and
 * per layer.  The getter returns the current form (negative on a bad width).
 * msur_conv_set_persistent / msur_conv_get_persistent set and read bit 0 alone. */
int msur_conv_set_form(int bn, int form);
int msur_conv_get_form(int bn);
int msur_conv_set_persistent(int bn, int on);
int msur_conv_get_persistent(int bn);

/* Weight gradient of that convolution, ADDED to dw [Cout][taps][Cin] (FP32):
 *   dw[n][t][c] += sum_{b, l} dz[b, l, n] * x[b, l + t - (taps - 1) / 2, c]
 * taps 1 or 3; the position range is split over `splits` CTAs per tile (0 = enough to fill the
 * GPU), whose partial sums are added with atomics. */
int msur_conv_wgrad(const void* x, const void* dz, int B, int L, int Cin, int Cout, int taps, float* dw, int splits,
                    void* stream);

/* y[b, l, c] = (x[b, 2l, c] + x[b, 2l + 1, c]) / 2 for l < Lout (average pooling by two). */
int msur_pool2(const void* x, int B, int Lout, int C, void* y, void* stream);
/* Gradient into a SiLU output used twice, by the pooling and as a skip connection:
 *   dz[b, l, c] = (dpool[b, l / 2, c] / 2 + dcat[b, l, cat_off + c]) * silu'(z[b, l, c])
 * (dpool has Lp positions; either gradient may be NULL). */
int msur_skip_grad(const void* dpool, int Lp, const void* dcat, int cat_stride, int cat_off, const void* z, int B,
                   int L, int C, void* dz, void* stream);
/* out[b, l, :] = concat(x[b, l / 2, 0:C1], skip[b, l, 0:C2]): nearest upsampling by two and the
 * skip connection. */
int msur_upcat(const void* x, const void* skip, int B, int L, int C1, int C2, void* out, void* stream);
/* dz[b, l, c] = (dcat[b, 2l, c] + dcat[b, 2l + 1, c]) * silu'(z[b, l, c]) for l < Lh, c < C1
 * (dcat has C channels): the gradient through msur_upcat's upsampled half. */
int msur_upcat_bwd(const void* dcat, const void* z, int B, int Lh, int C1, int C, void* dz, void* stream);
/* db[c] += sum over rows of dz[row * stride + c]. */
int msur_bias_grad(const void* dz, uint64_t rows, int C, int stride, float* db, void* stream);
/* *loss += sum (pred - target)^2 over the first n_valid channels of each row (FP64 sums);
 * dp[row, c] = scale * (pred - target) (BF16, 0 in the padded channels up to dstride) when dp
 * is not NULL. */
int msur_mse(const float* pred, int pstride, const float* target, int tstride, uint64_t rows, int n_valid, void* dp,
             int dstride, float scale, double* loss, void* stream);
/* One Adam step with decoupled weight decay (FP32 masters p, moments m, v; gradient g * gscale);
 * writes the BF16 copy p_bf16 when not NULL. */
int msur_adam(float* p, const float* g, float* m, float* v, uint64_t n, float lr, float b1, float b2, float eps,
              float wd, int step, float gscale, void* p_bf16, void* stream);
/* wt[c][t][n] = w[n][taps - 1 - t][c]: the weights of the data gradient. */
int msur_weight_transpose(const void* w, int N, int taps, int C, void* wt, void* stream);
/* Network input: x[b, l, 0:4] = track[b][0:4][l] (occupancy, + motifs, - motifs, LEF density),
 * x[b, l, 4:8] = params[b][0:4], the other C - 8 channels zero. */
int msur_assemble_input(const float* track, const float* params, int B, int L, int C, void* x, void* stream);
/* Training target of a band summed over cells (column-major uint32 [ncols][nrows], the
 * reference's ContactMatrixDense layout): out[j][d] = log1p(band[j][d] * nrows / sum_d band[j][d])
 * per bin j (0 for a bin without contacts), computed in FP64 and stored as FP32. */
int msur_band_target(const uint32_t* band, uint64_t ncols, int nrows, float* out, void* stream);
/* Per-map sums for Pearson r and relative L2 (FP64, ADDED to out[6 * m .. 6 * m + 5]) over the n
 * values of map m: sum p', sum r', sum p'^2, sum r'^2, sum p' r', sum (p - r)^2, where p' = p and
 * r' = r when means is NULL and p' = p - means[2m], r' = r - means[2m + 1] otherwise (the second
 * pass of the reference's two-pass Pearson, src/stats/correlation_impl.hpp:66-87). */
int msur_map_sums(const float* pred, uint64_t pstride_map, const float* ref, uint64_t rstride_map, uint64_t n,
                  int nmaps, const double* means, double* out, void* stream);
/* out[r][c] = in[r * stride + c] for c < n_valid (drop the padded channels of the head). */
int msur_compact_rows(const float* in, int stride, uint64_t rows, int n_valid, float* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MGPU_SURROGATE_H */
