// Kernels of the learned upsampler (a 3-level BF16 U-Net): 3x3 convolution
// forward / data-gradient as implicit GEMM and weight-gradient as a GEMM over
// pixels, both on the tensor cores (mma.sync m16n8k16 BF16 -> FP32), plus the
// element-wise layers, the L1 + SSIM loss and Adam. Activations are NHWC
// BF16 with channel counts that are multiples of 16.
//
// Conv layout: in [N][H][W][Cin], weights [Cout][3][3][Cin], out [N][H][W][Cout].
// The data gradient is a convolution of the output gradient with the weights
// flipped in space and transposed in channels (host-prepared).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vrc_nn.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr float LEAK = 0.05f;  // slope of the leaky ReLU for negative inputs

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------------------
// Forward 3x3 convolution (stride 1, zero padding 1).
// CTA: an output tile of TH rows x 16 columns, all COUT channels; 8 warps,
// warp w owns output rows w * RPW .. w * RPW + RPW - 1 (one m16 tile per row).
// Per 16-channel input chunk the CTA stages the (TH+2) x 18 input halo and the
// 9 x COUT x 16 weights in shared memory (rows padded to 24 BF16 so ldmatrix
// rows fall on distinct banks), then runs 9 taps x COUT/8 MMAs per m-tile.
constexpr int PIX_PAD = 24;  // bf16 per staged pixel / weight row (16 used)

// Optional fused input [up2(A) | B]: channels [0, Ca) come from A at half
// resolution (nearest 2x upsample on load) and [Ca, Ca + Cb) from B; Cin =
// Ca + Cb and `in` is A. With in_b == nullptr the input is `in` as is.
template <int COUT, int RPW>
__global__ void __launch_bounds__(256) conv3x3_fwd_kernel(const __nv_bfloat16* __restrict__ in, int N, int H, int W,
                                                          int Cin, const __nv_bfloat16* __restrict__ wt,
                                                          const float* __restrict__ bias, int relu, void* out,
                                                          int out_f32, const __nv_bfloat16* __restrict__ in_b,
                                                          int Ca) {
    constexpr int TH = 8 * RPW;
    constexpr int NT = COUT / 8;
    extern __shared__ __align__(16) __nv_bfloat16 smem[];
    __nv_bfloat16* s_in = smem;                                   // [TH+2][18][PIX_PAD]
    __nv_bfloat16* s_w = smem + (TH + 2) * 18 * PIX_PAD;          // [9][COUT][PIX_PAD]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * 16, y0 = blockIdx.y * TH, n = blockIdx.z;
    float acc[RPW][NT][4];
#pragma unroll
    for (int r = 0; r < RPW; ++r)
#pragma unroll
        for (int j = 0; j < NT; ++j) acc[r][j][0] = acc[r][j][1] = acc[r][j][2] = acc[r][j][3] = 0.f;

    for (int c0 = 0; c0 < Cin; c0 += 16) {
        // stage the input halo: (TH+2) x 18 pixels x 16 channels, 2 x 16 B per pixel
        for (int i = tid; i < (TH + 2) * 18 * 2; i += 256) {
            const int half = i & 1, pix = i >> 1;
            const int ry = pix / 18, rx = pix % 18;
            const int gy = y0 + ry - 1, gx = x0 + rx - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
                if (in_b == nullptr) {
                    v = *reinterpret_cast<const uint4*>(in + (((size_t)n * H + gy) * W + gx) * Cin + c0 + half * 8);
                } else if (c0 < Ca) {
                    const int Hh = H >> 1, Wh = W >> 1;
                    v = *reinterpret_cast<const uint4*>(in + (((size_t)n * Hh + (gy >> 1)) * Wh + (gx >> 1)) * Ca + c0 +
                                                        half * 8);
                } else {
                    const int Cb = Cin - Ca;
                    v = *reinterpret_cast<const uint4*>(in_b + (((size_t)n * H + gy) * W + gx) * Cb + (c0 - Ca) +
                                                        half * 8);
                }
            }
            *reinterpret_cast<uint4*>(s_in + (ry * 18 + rx) * PIX_PAD + half * 8) = v;
        }
        // stage weights [tap][cout][16]
        for (int i = tid; i < 9 * COUT * 2; i += 256) {
            const int half = i & 1, row = i >> 1;  // row = tap * COUT + co
            const int tap = row / COUT, co = row % COUT;
            const uint4 v = *reinterpret_cast<const uint4*>(wt + ((size_t)co * 9 + tap) * Cin + c0 + half * 8);
            *reinterpret_cast<uint4*>(s_w + row * PIX_PAD + half * 8) = v;
        }
        __syncthreads();
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int kh = tap / 3, kw = tap % 3;
            uint32_t a[RPW][4];
#pragma unroll
            for (int r = 0; r < RPW; ++r) {
                const int row = warp * RPW + r + kh;
                const __nv_bfloat16* p = s_in + (row * 18 + kw + (lane & 15)) * PIX_PAD + (lane >> 4) * 8;
                ldsm_x4(smem_u32(p), a[r][0], a[r][1], a[r][2], a[r][3]);
            }
#pragma unroll
            for (int j = 0; j < NT; j += 2) {
                // two n-tiles: lanes 0-15 -> tile j (k 0 / 8), lanes 16-31 -> tile j + 1
                const int jj = j + (lane >> 4);
                const int co = (jj < NT ? jj : j) * 8 + (lane & 7);
                const __nv_bfloat16* p = s_w + (tap * COUT + co) * PIX_PAD + ((lane >> 3) & 1) * 8;
                uint32_t b0, b1, b2, b3;
                ldsm_x4(smem_u32(p), b0, b1, b2, b3);
#pragma unroll
                for (int r = 0; r < RPW; ++r) {
                    mma_bf16(acc[r][j], a[r][0], a[r][1], a[r][2], a[r][3], b0, b1);
                    if (j + 1 < NT) mma_bf16(acc[r][j + 1], a[r][0], a[r][1], a[r][2], a[r][3], b2, b3);
                }
            }
        }
        __syncthreads();
    }
    // epilogue: bias, optional ReLU, store (d0,d1: pixel g; d2,d3: pixel g + 8)
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int y = y0 + warp * RPW + r;
        if (y >= H) continue;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int co = j * 8 + 2 * t;
            const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = x0 + g + 8 * h;
                if (x >= W) continue;
                float v0 = acc[r][j][2 * h] + b0, v1 = acc[r][j][2 * h + 1] + b1;
                if (relu == 1) {
                    v0 = fmaxf(v0, 0.f);
                    v1 = fmaxf(v1, 0.f);
                } else if (relu == 2) {  // leaky ReLU
                    v0 = v0 > 0.f ? v0 : LEAK * v0;
                    v1 = v1 > 0.f ? v1 : LEAK * v1;
                }
                const size_t o = (((size_t)n * H + y) * W + x) * COUT + co;
                if (out_f32) {
                    *reinterpret_cast<float2*>(static_cast<float*>(out) + o) = make_float2(v0, v1);
                } else {
                    *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(out) + o) =
                        __floats2bfloat162_rn(v0, v1);
                }
            }
        }
    }
}

template <int COUT, int RPW>
cudaError_t conv_fwd_t(const __nv_bfloat16* in, int N, int H, int W, int Cin, const __nv_bfloat16* w,
                       const float* bias, int relu, void* out, int out_f32, cudaStream_t s,
                       const __nv_bfloat16* in_b = nullptr, int Ca = 0) {
    constexpr int TH = 8 * RPW;
    const size_t smem = ((TH + 2) * 18 * PIX_PAD + 9 * COUT * PIX_PAD) * sizeof(__nv_bfloat16);
    auto k = conv3x3_fwd_kernel<COUT, RPW>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((W + 15) / 16, (H + TH - 1) / TH, N);
    k<<<grid, 256, smem, s>>>(in, N, H, W, Cin, w, bias, relu, out, out_f32, in_b, Ca);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Weight gradient: dW[co][tap][ci] += sum_p dout[p][co] * in[p + tap - 1][ci]
// (and dbias[co] += sum_p dout[p][co] when requested).
// CTA: one tap, all COUT output channels, a 64-channel input block, and a
// run of PIX_TILES 8x16 pixel tiles; per tile it stages dout (128 x COUT) and
// the shifted input (128 x 64), rows padded to stride+8 BF16, and runs
// 8 k-steps of 16 pixels: A = dout^T via ldmatrix.trans, B = input via
// ldmatrix.trans. Partial sums are added to the FP32 gradients atomically.
constexpr int WG_CI = 64;

template <int COUT>
__global__ void __launch_bounds__(256) conv3x3_wgrad_kernel(const __nv_bfloat16* __restrict__ in,
                                                            const __nv_bfloat16* __restrict__ dout, int N, int H,
                                                            int W, int Cin, float* dw, float* dbias,
                                                            int tiles_per_cta) {
    constexpr int MT = COUT / 16;               // m16 tiles along COUT
    constexpr int NG = 8 / MT;                  // warps sharing one m tile, each owns 8/NG n-tiles
    constexpr int NTW = (WG_CI / 8) / NG;       // n8 tiles per warp
    constexpr int DS = COUT + 8, IS = WG_CI + 8;  // padded row strides (bf16)
    extern __shared__ __align__(16) __nv_bfloat16 smem[];
    __nv_bfloat16* s_d = smem;                  // [128][DS]
    __nv_bfloat16* s_i = smem + 128 * DS;       // [128][IS]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tap = blockIdx.y, kh = tap / 3, kw = tap % 3;
    const int ci0 = blockIdx.z * WG_CI;
    const int mt = warp % MT, ng = warp / MT;
    const int tiles_x = (W + 15) / 16, tiles_y = (H + 7) / 8, ntiles = tiles_x * tiles_y * N;
    float acc[NTW][4];
#pragma unroll
    for (int j = 0; j < NTW; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    float bsum = 0.f;
    const int t_begin = blockIdx.x * tiles_per_cta, t_end = min(ntiles, t_begin + tiles_per_cta);
    for (int tile = t_begin; tile < t_end; ++tile) {
        const int n = tile / (tiles_x * tiles_y), rem = tile % (tiles_x * tiles_y);
        const int y0 = (rem / tiles_x) * 8, x0 = (rem % tiles_x) * 16;
        // stage dout rows (128 pixels x COUT) and shifted input (128 x 64)
        for (int i = tid; i < 128 * (COUT / 8); i += 256) {
            const int p = i / (COUT / 8), v8 = i % (COUT / 8);
            const int y = y0 + p / 16, x = x0 + p % 16;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (y < H && x < W) v = *reinterpret_cast<const uint4*>(dout + (((size_t)n * H + y) * W + x) * COUT + v8 * 8);
            *reinterpret_cast<uint4*>(s_d + p * DS + v8 * 8) = v;
        }
        for (int i = tid; i < 128 * (WG_CI / 8); i += 256) {
            const int p = i / (WG_CI / 8), v8 = i % (WG_CI / 8);
            const int y = y0 + p / 16, x = x0 + p % 16;
            const int gy = y + kh - 1, gx = x + kw - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (y < H && x < W && gy >= 0 && gy < H && gx >= 0 && gx < W && ci0 + v8 * 8 < Cin)
                v = *reinterpret_cast<const uint4*>(in + (((size_t)n * H + gy) * W + gx) * Cin + ci0 + v8 * 8);
            *reinterpret_cast<uint4*>(s_i + p * IS + v8 * 8) = v;
        }
        __syncthreads();
        if (dbias && tap == 0 && blockIdx.z == 0)
            for (int co = tid; co < COUT; co += 256)
                for (int p = 0; p < 128; ++p) bsum += __bfloat162float(s_d[p * DS + co]);
#pragma unroll
        for (int k0 = 0; k0 < 128; k0 += 16) {
            // A (m = co, k = pixel): stored [pixel][co] -> ldmatrix.trans
            uint32_t a0, a1, a2, a3;
            {
                const int p = k0 + ((lane >> 4) << 3) + (lane & 7);
                const int co = mt * 16 + ((lane >> 3) & 1) * 8;
                ldsm_x4_t(smem_u32(s_d + p * DS + co), a0, a1, a2, a3);
            }
#pragma unroll
            for (int j = 0; j < NTW; j += 2) {
                // B (k = pixel, n = ci): stored [pixel][ci] -> ldmatrix.trans; two n-tiles
                const int nt = ng * NTW + j + (lane >> 4);
                const int p = k0 + ((lane >> 3) & 1) * 8 + (lane & 7);
                uint32_t b0, b1, b2, b3;
                ldsm_x4_t(smem_u32(s_i + p * IS + nt * 8), b0, b1, b2, b3);
                mma_bf16(acc[j], a0, a1, a2, a3, b0, b1);
                if (j + 1 < NTW) mma_bf16(acc[j + 1], a0, a1, a2, a3, b2, b3);
            }
        }
        __syncthreads();
    }
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < NTW; ++j) {
        const int ci = ci0 + (ng * NTW + j) * 8 + 2 * t;
        const int co = mt * 16 + g;
        if (ci < Cin) {
            atomicAdd(dw + ((size_t)co * 9 + tap) * Cin + ci, acc[j][0]);
            atomicAdd(dw + ((size_t)co * 9 + tap) * Cin + ci + 1, acc[j][1]);
            atomicAdd(dw + ((size_t)(co + 8) * 9 + tap) * Cin + ci, acc[j][2]);
            atomicAdd(dw + ((size_t)(co + 8) * 9 + tap) * Cin + ci + 1, acc[j][3]);
        }
    }
    if (dbias && tap == 0 && blockIdx.z == 0)
        for (int co = tid; co < COUT; co += 256) atomicAdd(dbias + co, bsum);
}

template <int COUT>
cudaError_t conv_wgrad_t(const __nv_bfloat16* in, const __nv_bfloat16* dout, int N, int H, int W, int Cin, float* dw,
                         float* dbias, cudaStream_t s) {
    const size_t smem = (128 * (COUT + 8) + 128 * (WG_CI + 8)) * sizeof(__nv_bfloat16);
    auto k = conv3x3_wgrad_kernel<COUT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int ntiles = ((W + 15) / 16) * ((H + 7) / 8) * N;
    const int per = 32;
    dim3 grid((ntiles + per - 1) / per, 9, (Cin + WG_CI - 1) / WG_CI);
    k<<<grid, 256, smem, s>>>(in, dout, N, H, W, Cin, dw, dbias, per);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// element-wise layers
// dy *= d relu / dx, read from the activation's sign (leaky: slope LEAK)
__global__ void relu_bwd_kernel(const __nv_bfloat16* y, __nv_bfloat16* dy, long long n, int leaky) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[i]) > 0.f))
            dy[i] = __float2bfloat16(leaky ? LEAK * __bfloat162float(dy[i]) : 0.f);
}

// 2x2 average pool times `scale`, NHWC (H, W even); scale 4 gives the
// sum-pooling that is the backward of the nearest 2x upsample
__global__ void avgpool_kernel(const __nv_bfloat16* in, int N, int H, int W, int C, float scale, __nv_bfloat16* out) {
    const int Ho = H / 2, Wo = W / 2;
    const long long n = (long long)N * Ho * Wo * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long long r = i / C;
        const int x = (int)(r % Wo), y = (int)((r / Wo) % Ho), b = (int)(r / ((long long)Wo * Ho));
        const __nv_bfloat16* p = in + (((size_t)b * H + 2 * y) * W + 2 * x) * C + c;
        const float s = __bfloat162float(p[0]) + __bfloat162float(p[C]) + __bfloat162float(p[(size_t)W * C]) +
                        __bfloat162float(p[(size_t)W * C + C]);
        out[i] = __float2bfloat16(0.25f * scale * s);
    }
}
// backward of avgpool: din = dout / 4 replicated; with `scale` = 1 it is the
// nearest 2x upsample (whose backward is sum-pooling: avgpool * 4)
__global__ void upsample2_kernel(const __nv_bfloat16* in, int N, int H, int W, int C, float scale,
                                 __nv_bfloat16* out) {
    const int Ho = 2 * H, Wo = 2 * W;
    const long long n = (long long)N * Ho * Wo * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long long r = i / C;
        const int x = (int)(r % Wo), y = (int)((r / Wo) % Ho), b = (int)(r / ((long long)Wo * Ho));
        out[i] = __float2bfloat16(scale * __bfloat162float(in[(((size_t)b * H + y / 2) * W + x / 2) * C + c]));
    }
}
// out[..., 0:Ca] = a, out[..., Ca:Ca+Cb] = b (and the split for the backward)
__global__ void concat_kernel(const __nv_bfloat16* a, int Ca, const __nv_bfloat16* b, int Cb, long long npix,
                              __nv_bfloat16* out, int split) {
    const int C = Ca + Cb;
    const long long n = npix * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / C;
        const int c = (int)(i % C);
        if (!split) {
            out[i] = c < Ca ? a[p * Ca + c] : b[p * Cb + c - Ca];
        } else {  // out is the source gradient; a, b receive its halves
            if (c < Ca) const_cast<__nv_bfloat16*>(a)[p * Ca + c] = out[i];
            else const_cast<__nv_bfloat16*>(b)[p * Cb + c - Ca] = out[i];
        }
    }
}
__global__ void add_bf16_kernel(__nv_bfloat16* a, const __nv_bfloat16* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] = __float2bfloat16(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}

// Upsampler head: 16 channels at H x W -> 4 channels at 2H x 2W (depth to
// space, channel c = 4 * (2 * dy + dx) + k) plus the bilinear 2x upsample of
// the low-resolution colour `base` (NHWC float, 4 channels) as a residual.
__device__ __forceinline__ float bilerp_base(const float* base, int b, int H, int W, int oy, int ox, int k) {
    // align-corners = false: source coordinate (o + 0.5) / 2 - 0.5
    const float sy = fmaxf((oy + 0.5f) * 0.5f - 0.5f, 0.f), sx = fmaxf((ox + 0.5f) * 0.5f - 0.5f, 0.f);
    const int y0 = min((int)sy, H - 1), x0 = min((int)sx, W - 1);
    const int y1 = min(y0 + 1, H - 1), x1 = min(x0 + 1, W - 1);
    const float fy = sy - y0, fx = sx - x0;
    const float* p = base + (size_t)b * H * W * 4;
    const float v00 = p[((size_t)y0 * W + x0) * 4 + k], v01 = p[((size_t)y0 * W + x1) * 4 + k];
    const float v10 = p[((size_t)y1 * W + x0) * 4 + k], v11 = p[((size_t)y1 * W + x1) * 4 + k];
    return (v00 * (1.f - fx) + v01 * fx) * (1.f - fy) + (v10 * (1.f - fx) + v11 * fx) * fy;
}
__global__ void head_fwd_kernel(const float* feat16, const float* base, int N, int H, int W, float* out) {
    const int Ho = 2 * H, Wo = 2 * W;
    const long long n = (long long)N * Ho * Wo * 4;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i & 3);
        const long long r = i >> 2;
        const int ox = (int)(r % Wo), oy = (int)((r / Wo) % Ho), b = (int)(r / ((long long)Wo * Ho));
        const int c = 4 * (2 * (oy & 1) + (ox & 1)) + k;
        const float f = feat16[(((size_t)b * H + oy / 2) * W + ox / 2) * 16 + c];
        out[i] = f + bilerp_base(base, b, H, W, oy, ox, k);
    }
}
// gradient of the head w.r.t. feat16 (BF16, for the conv backward)
__global__ void head_bwd_kernel(const float* dout, int N, int H, int W, __nv_bfloat16* dfeat16) {
    const long long n = (long long)N * H * W * 16;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % 16);
        const long long r = i / 16;
        const int x = (int)(r % W), y = (int)((r / W) % H), b = (int)(r / ((long long)W * H));
        const int k = c & 3, q = c >> 2, dy = q >> 1, dx = q & 1;
        const int oy = 2 * y + dy, ox = 2 * x + dx;
        dfeat16[i] = __float2bfloat16(dout[(((size_t)b * 2 * H + oy) * 2 * W + ox) * 4 + k]);
    }
}
__global__ void bilinear_up_kernel(const float* base, int N, int H, int W, float* out) {
    const int Ho = 2 * H, Wo = 2 * W;
    const long long n = (long long)N * Ho * Wo * 4;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i & 3);
        const long long r = i >> 2;
        const int ox = (int)(r % Wo), oy = (int)((r / Wo) % Ho), b = (int)(r / ((long long)Wo * Ho));
        out[i] = bilerp_base(base, b, H, W, oy, ox, k);
    }
}

// ---------------------------------------------------------------------------
// Loss: mean over pixels/channels of  |x - y| + lambda * (1 - SSIM(x, y)),
// SSIM on R x R box windows (R = 2r+1, clamped at borders) per channel.
// Pass 1 writes per-window statistics' derivative coefficients, pass 2 sums
// them over the windows covering each pixel to form dL/dx.
constexpr float SSIM_C1 = 0.0001f, SSIM_C2 = 0.0009f;  // (0.01)^2, (0.03)^2

__global__ void ssim_coef_kernel(const float* x, const float* y, int N, int H, int W, int r, float* coef,
                                 float* loss_acc) {
    const long long n = (long long)N * H * W * 4;
    float lsum = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i & 3);
        const long long pix = i >> 2;
        const int px = (int)(pix % W), py = (int)((pix / W) % H), b = (int)(pix / ((long long)W * H));
        float sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
        int cnt = 0;
        for (int dy = -r; dy <= r; ++dy) {
            const int yy = py + dy;
            if (yy < 0 || yy >= H) continue;
            for (int dx = -r; dx <= r; ++dx) {
                const int xx = px + dx;
                if (xx < 0 || xx >= W) continue;
                const size_t o = (((size_t)b * H + yy) * W + xx) * 4 + k;
                const float a = x[o], c = y[o];
                sx += a;
                sy += c;
                sxx += a * a;
                syy += c * c;
                sxy += a * c;
                ++cnt;
            }
        }
        const float inv = 1.f / cnt;
        const float mx = sx * inv, my = sy * inv;
        const float vx = sxx * inv - mx * mx, vy = syy * inv - my * my, cxy = sxy * inv - mx * my;
        const float A1 = 2 * mx * my + SSIM_C1, A2 = 2 * cxy + SSIM_C2;
        const float B1 = mx * mx + my * my + SSIM_C1, B2 = vx + vy + SSIM_C2;
        const float S = (A1 * A2) / (B1 * B2);
        lsum += S;
        // dS/dx_q = inv * (alpha + beta * x_q + gamma * y_q) for q in the window
        // partials holding the (biased) variance / covariance fixed; their own
        // dependence on x_q enters through d vx/d x_q and d cxy/d x_q below
        const float dS_dmx = (2 * my * A2) / (B1 * B2) - S * (2 * mx) / B1;
        // d vx/d x_q = 2 (x_q - mx)/cnt ; d cxy/d x_q = (y_q - my)/cnt ; d mx/d x_q = 1/cnt
        const float dS_dvx = -S / B2;
        const float dS_dcxy = 2 * A1 / (B1 * B2);
        // dS/dx_q = inv * [dS_dmx + dS_dvx * 2 (x_q - mx) + dS_dcxy * (y_q - my)]
        float* cf = coef + (size_t)i * 3;
        cf[0] = inv * (dS_dmx - 2 * dS_dvx * mx - dS_dcxy * my);
        cf[1] = inv * (2 * dS_dvx);
        cf[2] = inv * dS_dcxy;
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(FULL, lsum, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc + 1, lsum);
}

__global__ void loss_grad_kernel(const float* x, const float* y, int N, int H, int W, int r, const float* coef,
                                 float lambda, float inv_count, float* dx, float* loss_acc) {
    const long long n = (long long)N * H * W * 4;
    float lsum = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i & 3);
        const long long pix = i >> 2;
        const int px = (int)(pix % W), py = (int)((pix / W) % H), b = (int)(pix / ((long long)W * H));
        const float xv = x[i], yv = y[i];
        float a = 0, bb = 0, c = 0;
        for (int dy = -r; dy <= r; ++dy) {
            const int yy = py + dy;
            if (yy < 0 || yy >= H) continue;
            for (int ddx = -r; ddx <= r; ++ddx) {
                const int xx = px + ddx;
                if (xx < 0 || xx >= W) continue;
                const float* cf = coef + ((((size_t)b * H + yy) * W + xx) * 4 + k) * 3;
                a += cf[0];
                bb += cf[1];
                c += cf[2];
            }
        }
        const float dssim = a + bb * xv + c * yv;  // d(sum_w S_w)/dx_i
        const float d = xv - yv;
        lsum += fabsf(d);
        dx[i] = inv_count * ((d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f)) - lambda * dssim);
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(FULL, lsum, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc, lsum);
}

// Adam on FP32 master weights; writes the BF16 copy used by the convolutions.
__global__ void adam_kernel(float* w, const float* g, float* m, float* v, __nv_bfloat16* w_bf16, long long n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (w_bf16) w_bf16[i] = __float2bfloat16(wi);
    }
}

// Data-gradient weights: wt[ci][kh][kw][co] = w[co][2-kh][2-kw][ci].
__global__ void flip_weights_kernel(const __nv_bfloat16* w, int Cout, int Cin, __nv_bfloat16* wt) {
    const long long n = (long long)Cout * 9 * Cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int co = (int)(i % Cout);
        const long long r = i / Cout;
        const int tap = (int)(r % 9), ci = (int)(r / 9);
        wt[i] = w[((size_t)co * 9 + (8 - tap)) * Cin + ci];
    }
}

// Network input: RGBA colour + first-hit depth + gradient magnitude of the
// low-resolution march, packed NHWC BF16 with 16 channels (10 zero).
__global__ void pack_input_kernel(const float* rgba, const float* aux2, long long npix, __nv_bfloat16* out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        __nv_bfloat16 v[16];
        for (int c = 0; c < 4; ++c) v[c] = __float2bfloat16(rgba[p * 4 + c]);
        v[4] = __float2bfloat16(aux2 ? aux2[p * 2] : 0.f);
        v[5] = __float2bfloat16(aux2 ? aux2[p * 2 + 1] : 0.f);
        for (int c = 6; c < 16; ++c) v[c] = __float2bfloat16(0.f);
        uint4* o = reinterpret_cast<uint4*>(out + p * 16);
        o[0] = *reinterpret_cast<uint4*>(&v[0]);
        o[1] = *reinterpret_cast<uint4*>(&v[8]);
    }
}

// Mean alpha of each tile x tile block of an RGBA FP32 image (the content
// map that picks the probe tile); one CTA per block, ny x nx blocks.
__global__ void tile_alpha_kernel(const float* rgba, int H, int W, int tile, int nx, float* out) {
    const int bx = blockIdx.x % nx, by = blockIdx.x / nx;
    float s = 0.f;
    for (int i = threadIdx.x; i < tile * tile; i += blockDim.x) {
        const int x = bx * tile + i % tile, y = by * tile + i / tile;
        if (x < W && y < H) s += rgba[((size_t)y * W + x) * 4 + 3];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        out[blockIdx.x] = t / float(tile * tile);
    }
}

// Probe: squared error sum and max |a - b| over a pixel window of two RGBA
// FP32 images of width W (a: the network's frame, b: the plain render).
__global__ void probe_error_kernel(const float* a, const float* b, int W, int x0, int y0, int w, int h, float* out2) {
    float se = 0.f, mx = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h * 4; i += gridDim.x * blockDim.x) {
        const int k = i & 3, p = i >> 2;
        const size_t o = ((size_t)(y0 + p / w) * W + (x0 + p % w)) * 4 + k;
        const float d = fminf(fmaxf(a[o], 0.f), 1.f) - fminf(fmaxf(b[o], 0.f), 1.f);
        se += d * d;
        mx = fmaxf(mx, fabsf(d));
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_xor_sync(FULL, se, o);
        mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out2, se);
        atomicMax(reinterpret_cast<int*>(out2 + 1), __float_as_int(mx));  // non-negative floats order as ints
    }
}

int ew_grid(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

int status_of(cudaError_t e) { return e == cudaSuccess ? 0 : 2; }

}  // namespace

extern "C" {

int vrc_nn_conv3x3_fwd(const void* in, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout,
                       int relu, void* out, int out_f32, void* stream) {
    if (!in || !w || !out || N < 1 || H < 1 || W < 1 || Cin < 16 || Cin % 16) return 1;
    const auto* i = static_cast<const __nv_bfloat16*>(in);
    const auto* wt = static_cast<const __nv_bfloat16*>(w);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (Cout) {
        case 16: return status_of(conv_fwd_t<16, 2>(i, N, H, W, Cin, wt, bias, relu, out, out_f32, s));
        case 32: return status_of(conv_fwd_t<32, 2>(i, N, H, W, Cin, wt, bias, relu, out, out_f32, s));
        case 64: return status_of(conv_fwd_t<64, 2>(i, N, H, W, Cin, wt, bias, relu, out, out_f32, s));
        case 128: return status_of(conv_fwd_t<128, 1>(i, N, H, W, Cin, wt, bias, relu, out, out_f32, s));
        default: return 4;
    }
}

int vrc_nn_conv3x3_fwd_upcat(const void* a, int Ca, const void* b, int Cb, int N, int H, int W, const void* w,
                             const float* bias, int Cout, int relu, void* out, int out_f32, void* stream) {
    if (!a || !b || !w || !out || N < 1 || H < 2 || W < 2 || H % 2 || W % 2 || Ca < 16 || Ca % 16 || Cb < 16 ||
        Cb % 16)
        return 1;
    const auto* ia = static_cast<const __nv_bfloat16*>(a);
    const auto* ib = static_cast<const __nv_bfloat16*>(b);
    const auto* wt = static_cast<const __nv_bfloat16*>(w);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int Cin = Ca + Cb;
    switch (Cout) {
        case 16: return status_of(conv_fwd_t<16, 2>(ia, N, H, W, Cin, wt, bias, relu, out, out_f32, s, ib, Ca));
        case 32: return status_of(conv_fwd_t<32, 2>(ia, N, H, W, Cin, wt, bias, relu, out, out_f32, s, ib, Ca));
        case 64: return status_of(conv_fwd_t<64, 2>(ia, N, H, W, Cin, wt, bias, relu, out, out_f32, s, ib, Ca));
        case 128: return status_of(conv_fwd_t<128, 1>(ia, N, H, W, Cin, wt, bias, relu, out, out_f32, s, ib, Ca));
        default: return 4;
    }
}

int vrc_nn_conv3x3_wgrad(const void* in, const void* dout, int N, int H, int W, int Cin, int Cout, float* dw,
                         float* dbias, void* stream) {
    if (!in || !dout || !dw || N < 1 || H < 1 || W < 1 || Cin < 16 || Cin % 16) return 1;
    const auto* i = static_cast<const __nv_bfloat16*>(in);
    const auto* d = static_cast<const __nv_bfloat16*>(dout);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (Cout) {
        case 16: return status_of(conv_wgrad_t<16>(i, d, N, H, W, Cin, dw, dbias, s));
        case 32: return status_of(conv_wgrad_t<32>(i, d, N, H, W, Cin, dw, dbias, s));
        case 64: return status_of(conv_wgrad_t<64>(i, d, N, H, W, Cin, dw, dbias, s));
        case 128: return status_of(conv_wgrad_t<128>(i, d, N, H, W, Cin, dw, dbias, s));
        default: return 4;
    }
}

int vrc_nn_relu_bwd(const void* y, void* dy, long long n, int leaky, void* stream) {
    relu_bwd_kernel<<<ew_grid(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(y), static_cast<__nv_bfloat16*>(dy), n, leaky);
    return status_of(cudaGetLastError());
}

int vrc_nn_avgpool2(const void* in, int N, int H, int W, int C, float scale, void* out, void* stream) {
    if (H % 2 || W % 2) return 1;
    avgpool_kernel<<<ew_grid((long long)N * H * W * C / 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(in), N, H, W, C, scale, static_cast<__nv_bfloat16*>(out));
    return status_of(cudaGetLastError());
}

int vrc_nn_upsample2(const void* in, int N, int H, int W, int C, float scale, void* out, void* stream) {
    upsample2_kernel<<<ew_grid((long long)N * H * W * C * 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(in), N, H, W, C, scale, static_cast<__nv_bfloat16*>(out));
    return status_of(cudaGetLastError());
}

int vrc_nn_concat(const void* a, int Ca, const void* b, int Cb, long long npix, void* out, int split, void* stream) {
    concat_kernel<<<ew_grid(npix * (Ca + Cb)), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(a), Ca, static_cast<const __nv_bfloat16*>(b), Cb, npix,
        static_cast<__nv_bfloat16*>(out), split);
    return status_of(cudaGetLastError());
}

int vrc_nn_add(void* a, const void* b, long long n, void* stream) {
    add_bf16_kernel<<<ew_grid(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<__nv_bfloat16*>(a), static_cast<const __nv_bfloat16*>(b), n);
    return status_of(cudaGetLastError());
}

int vrc_nn_head_fwd(const float* feat16, const float* base, int N, int H, int W, float* out, void* stream) {
    head_fwd_kernel<<<ew_grid((long long)N * H * W * 16), 256, 0, static_cast<cudaStream_t>(stream)>>>(feat16, base, N,
                                                                                                       H, W, out);
    return status_of(cudaGetLastError());
}

int vrc_nn_head_bwd(const float* dout, int N, int H, int W, void* dfeat16, void* stream) {
    head_bwd_kernel<<<ew_grid((long long)N * H * W * 16), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        dout, N, H, W, static_cast<__nv_bfloat16*>(dfeat16));
    return status_of(cudaGetLastError());
}

int vrc_nn_bilinear_up2(const float* base, int N, int H, int W, float* out, void* stream) {
    bilinear_up_kernel<<<ew_grid((long long)N * H * W * 16), 256, 0, static_cast<cudaStream_t>(stream)>>>(base, N, H,
                                                                                                          W, out);
    return status_of(cudaGetLastError());
}

int vrc_nn_loss(const float* x, const float* y, int N, int H, int W, int radius, float lambda, float* coef_scratch,
                float* dx, float* loss2, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long n = (long long)N * H * W * 4;
    ssim_coef_kernel<<<ew_grid(n), 256, 0, s>>>(x, y, N, H, W, radius, coef_scratch, loss2);
    loss_grad_kernel<<<ew_grid(n), 256, 0, s>>>(x, y, N, H, W, radius, coef_scratch, lambda, 1.f / (float)n, dx,
                                                loss2);
    return status_of(cudaGetLastError());
}

int vrc_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, float lr, float b1, float b2,
                float eps, int step, void* stream) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<ew_grid(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, g, m, v,
                                                                          static_cast<__nv_bfloat16*>(w_bf16), n, lr,
                                                                          b1, b2, eps, c1, c2);
    return status_of(cudaGetLastError());
}

int vrc_nn_flip_weights(const void* w, int Cout, int Cin, void* wt, void* stream) {
    flip_weights_kernel<<<ew_grid((long long)Cout * 9 * Cin), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(w), Cout, Cin, static_cast<__nv_bfloat16*>(wt));
    return status_of(cudaGetLastError());
}

int vrc_nn_probe_error(const float* a, const float* b, int W, int x0, int y0, int w, int h, float* out2,
                       void* stream) {
    if (!a || !b || !out2 || w < 1 || h < 1) return 1;
    probe_error_kernel<<<16, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, b, W, x0, y0, w, h, out2);
    return status_of(cudaGetLastError());
}

int vrc_nn_pack_input(const float* rgba, const float* aux2, long long npix, void* out, void* stream) {
    pack_input_kernel<<<ew_grid(npix), 256, 0, static_cast<cudaStream_t>(stream)>>>(rgba, aux2, npix,
                                                                                   static_cast<__nv_bfloat16*>(out));
    return status_of(cudaGetLastError());
}

int vrc_nn_tile_alpha(const float* rgba, int H, int W, int tile, int ny, int nx, float* out, void* stream) {
    if (!rgba || !out || tile < 1 || ny < 1 || nx < 1) return 1;
    tile_alpha_kernel<<<ny * nx, 256, 0, static_cast<cudaStream_t>(stream)>>>(rgba, H, W, tile, nx, out);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // extern "C"
