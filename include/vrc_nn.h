/*
 * vrc_nn -- kernels of the learned upsampler (no counterpart in the reference).
 *
 * The learned form renders a half-resolution, half-rate march and rebuilds
 * the full-resolution frame with a 3-level BF16 U-Net (32/64/128 channels,
 * 3x3 convolutions, FP32 accumulation on the tensor cores). These are its
 * training and inference kernels; the network and its training loop are
 * driven from the host (voreen_gb300/learned.py). All pointers are device
 * pointers; tensors are NHWC; `stream` is a cudaStream_t. Return 0 on
 * success, 1 for invalid arguments, 2 for a CUDA error, 4 for an unsupported
 * channel count.
 */
#ifndef VRC_NN_H
#define VRC_NN_H
#ifdef __cplusplus
extern "C" {
#endif

/* out = act(conv3x3(in, w) + bias), act: 0 none, 1 ReLU, 2 leaky ReLU
 * (slope 0.05 below zero). in BF16 [N][H][W][Cin]
 * (Cin % 16 == 0), w BF16 [Cout][3][3][Cin], bias FP32 [Cout] (nullable),
 * Cout in {16, 32, 64, 128}; out BF16 or FP32 (out_f32) [N][H][W][Cout]. */
int vrc_nn_conv3x3_fwd(const void* in, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout,
                       int relu, void* out, int out_f32, void* stream);
/* Decoder form: the input is [nearest 2x upsample of a | b] built on load
 * (a: [N][H/2][W/2][Ca], b: [N][H][W][Cb]; Ca, Cb multiples of 16), so the
 * upsampled and concatenated tensor is never written. */
int vrc_nn_conv3x3_fwd_upcat(const void* a, int Ca, const void* b, int Cb, int N, int H, int W, const void* w,
                             const float* bias, int Cout, int relu, void* out, int out_f32, void* stream);
/* dw[co][kh][kw][ci] += sum over pixels of dout * shifted in (FP32), and
 * dbias[co] += sum of dout (nullable). */
int vrc_nn_conv3x3_wgrad(const void* in, const void* dout, int N, int H, int W, int Cin, int Cout, float* dw,
                         float* dbias, void* stream);
/* wt[ci][kh][kw][co] = w[co][2-kh][2-kw][ci]: weights for the data gradient,
 * which is vrc_nn_conv3x3_fwd(dout, wt). */
int vrc_nn_flip_weights(const void* w, int Cout, int Cin, void* wt, void* stream);
/* dy *= act'(x) read from the activation y (in place, BF16): 0 (ReLU) or
 * 0.05 (leaky) where y <= 0. */
int vrc_nn_relu_bwd(const void* y, void* dy, long long n, int leaky, void* stream);
/* 2x2 average pool times `scale` (4: sum pool). */
int vrc_nn_avgpool2(const void* in, int N, int H, int W, int C, float scale, void* out, void* stream);
/* nearest 2x upsample times `scale` (0.25: backward of the average pool). */
int vrc_nn_upsample2(const void* in, int N, int H, int W, int C, float scale, void* out, void* stream);
/* channel concat out = [a | b] (split != 0: the reverse, out -> a, b). */
int vrc_nn_concat(const void* a, int Ca, const void* b, int Cb, long long npix, void* out, int split, void* stream);
/* a += b, BF16. */
int vrc_nn_add(void* a, const void* b, long long n, void* stream);
/* Head: 16 FP32 channels at H x W -> 2H x 2W x 4 by depth-to-space, plus the
 * bilinear 2x upsample of the low-resolution RGBA `base` (FP32 NHWC). */
int vrc_nn_head_fwd(const float* feat16, const float* base, int N, int H, int W, float* out, void* stream);
int vrc_nn_head_bwd(const float* dout, int N, int H, int W, void* dfeat16, void* stream);
/* Bilinear 2x upsample of an RGBA FP32 image (the method without the network). */
int vrc_nn_bilinear_up2(const float* base, int N, int H, int W, float* out, void* stream);
/* L1 + lambda * (1 - SSIM) over RGBA FP32 images ((2r+1)^2 box windows):
 * writes dL/dx (mean normalisation) and adds [sum |x-y|, sum SSIM] to
 * loss2. coef_scratch holds 3 floats per element. */
int vrc_nn_loss(const float* x, const float* y, int N, int H, int W, int radius, float lambda, float* coef_scratch,
                float* dx, float* loss2, void* stream);
/* Adam step on FP32 master weights; refreshes the BF16 copy (nullable). */
int vrc_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, float lr, float b1, float b2,
                float eps, int step, void* stream);
/* Probe check: adds [sum of squared error, max |a-b|] over the window
 * (x0, y0, w, h) of two RGBA FP32 images of width W (values clamped to
 * [0,1]) to out2 (zeroed by the caller). */
int vrc_nn_probe_error(const float* a, const float* b, int W, int x0, int y0, int w, int h, float* out2,
                       void* stream);
/* Network input from a low-resolution march: RGBA FP32 + aux FP32x2 (first-hit
 * depth, gradient magnitude; nullable) -> BF16 NHWC with 16 channels. */
int vrc_nn_pack_input(const float* rgba, const float* aux2, long long npix, void* out, void* stream);

/* Mean alpha of each tile x tile block of an RGBA FP32 H x W image into
 * out[ny][nx] (the learned path's content map for choosing its probe tile). */
int vrc_nn_tile_alpha(const float* rgba, int H, int W, int tile, int ny, int nx, float* out, void* stream);

/* ---- inference on the 5th-generation tensor cores ------------------------ */

/* out = act(conv3x3([in0 | in1]) + bias) with tcgen05.mma on operands that
 * TMA stages in shared memory: input channels [0, C0) from in0, [C0, C0 + C1)
 * from in1 (C1 = 0: in0 only), both NHWC BF16 at N x H x W; C0, C1 multiples
 * of 16. wtc: the weights rearranged by vrc_nn_weights_tc with the same C0,
 * C1 and n_split (Cout / n_split output channels per CTA, a multiple of 16, at
 * most 128). out_mode 0: BF16 NHWC with act (0 none, 1 ReLU, 2 leaky); 1:
 * FP32 NHWC (act applied likewise). d_err (nullable): set non-zero by a CTA
 * whose bounded wait gave up (the output is then incomplete); the value names
 * the wait (1 weights, 2 free stage, 3 filled stage, 4 free accumulator,
 * 5 filled accumulator), and every non-zero value is a timeout
 * (VRC_ERR_TIMEOUT). The CTA then waits for its own copies and MMAs in flight,
 * frees its tensor memory and returns: no trap, and the next launch runs
 * normally. */
int vrc_nn_conv3x3_tc(const void* in0, int C0, const void* in1, int C1, int N, int H, int W, const void* wtc,
                      const float* bias, int Cout, int n_split, int act, void* out, int out_mode, int* d_err,
                      void* stream);
/* Limit of vrc_nn_conv3x3_tc's pipeline waits in nanoseconds of the global
 * timer, for launches made after the call (0 restores the default, 200 ms).
 * The waits for a CTA's own copies and MMAs in flight keep their fixed
 * 200 ms. A short limit makes the waits give up (d_err); used to exercise
 * that path. Returns 0. */
int vrc_nn_set_wait_limit(unsigned long long ns);
/* w BF16 [Cout][3][3][C0 + C1] -> the shared-memory operand image that
 * vrc_nn_conv3x3_tc loads (same size): per output-channel slice, tap and
 * channel chunk, a block of rows swizzled as the tensor cores read them. */
int vrc_nn_weights_tc(const void* w, int Cout, int C0, int C1, int n_split, void* wtc, void* stream);

#ifdef __cplusplus
}
#endif
#endif
