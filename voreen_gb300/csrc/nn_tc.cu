// Inference convolutions of the learned upsampler on the 5th-generation
// tensor cores: tcgen05.mma (BF16 x BF16 -> FP32 accumulators in tensor
// memory) with operands staged in shared memory by TMA.
//
// Activations are NHWC BF16. A stage holds one input row of CK channels (CK
// = 64, 32 or 16): a TMA box {CK channels, 130 pixels} from x0 - 1 lands as
// 130 rows of CK x 2 bytes with the 128-, 64- or 32-byte swizzle, which is the
// K-major swizzled tcgen05 operand layout (8-row groups 8 rows apart along M,
// K advanced inside a row by 32 bytes per MMA). The swizzle is a function of
// the shared-memory address, so moving the operand start by kx rows selects
// horizontal tap kx with no data movement: one row load serves the three taps
// of that row. The weights sit in shared memory in the same swizzled layout
// (rearranged once by vrc_nn_weights_tc).
//
// Tile: R output rows x 128 pixels (one MMA of M = 128 per row and tap) x
// n_tile output channels (N). The R + 2 input rows of the tile stream through
// the stages once, in channel chunks; each staged row feeds the up to three
// output rows (accumulators) it belongs to, so every input row is read once
// per tile rather than three times. Warp roles: 0 = TMA producer, 1 = MMA
// issuer and tensor-memory owner, 2..5 = epilogue (tensor memory -> bias,
// activation -> global). Two sets of R accumulators let the epilogue of one
// tile overlap the MMAs of the next. Every wait is bounded by %globaltimer:
// the pipeline waits by a host-settable limit (vrc_nn_set_wait_limit, 200 ms
// by default); on a timeout the CTA records an error code, waits for its own
// copies and MMAs in flight (bounded by a fixed 200 ms, whatever the pipeline
// limit, so no copy or MMA is left writing to memory the CTA gives back),
// frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "../../include/vrc_nn.h"

namespace {

constexpr int TM = 128;                 // output pixels per row tile (MMA M)
constexpr int HALO = TM + 2;            // input pixels a row tile reads (one staged row)
constexpr int MAX_STAGES = 8;
constexpr int MAX_ROWS = 4;             // output rows per tile
constexpr int EPI_WARPS = 4;
constexpr int THREADS = (2 + EPI_WARPS) * 32;
constexpr unsigned long long WAIT_NS = 200ull * 1000ull * 1000ull;
constexpr float LEAK = 0.05f;
constexpr int NBARS = 2 * MAX_STAGES + 2 + 2 + 2;  // full, empty, tmem full, tmem empty, weights, mma done
constexpr size_t SMEM_BUDGET = 224 * 1024;  // of the 227 KB a CTA may hold

struct TcParams {
    int N, H, W;
    int C0, C1, CK, nchunks;  // channels of map 0 / map 1, channels per K chunk, chunks per input row
    int n_tile, n_split, Cout;
    int rows;                 // output rows per tile (R)
    int stages;
    int act, out_mode;
    int tiles_x, tiles_y, pix_tiles;
    uint32_t tmem_cols;
    uint32_t row_bytes;       // CK * 2: bytes of one operand row (= the swizzle width)
    uint32_t layout;          // tcgen05 descriptor layout type of that swizzle
    uint32_t a_bytes, a_stride, b_bytes, b_stride;
    const float* bias;
    const uint8_t* wtc;
    void* out;
    int* err;
    unsigned long long wait_ns;  // limit of the pipeline waits
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of parity `parity` to complete; false after limit_ns or
// once another role has given up (abort flag in shared memory). sleep_ns > 0
// backs off between polls, leaving issue slots to the warps sharing the
// scheduler (the epilogue warps share theirs with the producer and the MMA
// issuer).
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, unsigned long long limit_ns,
                          unsigned sleep_ns = 0) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = gtime();
    for (;;) {
        for (int i = 0; i < 32; ++i) {
            if (mbar_try(bar, parity)) return true;
            if (sleep_ns) __nanosleep(sleep_ns);
        }
        if (abort_flag && *abort_flag) return false;
        if (gtime() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
                 : "memory");
}

// tcgen05 shared-memory operand descriptor of a K-major swizzled operand:
// start address, stride between 8-row groups (sbo), swizzle layout type
// (2: 128-byte, 4: 64-byte, 6: 32-byte); the leading offset is unused for
// K-major swizzled operands (field set to 1).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo, uint32_t layout) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
           (1ull << 46) | ((uint64_t)layout << 61);
}
// Instruction descriptor of kind::f16: FP32 accumulate, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float act_fn(float v, int act) {
    if (act == 1) return fmaxf(v, 0.f);
    if (act == 2) return v > 0.f ? v : LEAK * v;
    return v;
}

__device__ void record_error(int* err, volatile int* abort_flag, int code) {
    *abort_flag = 1;
    if (err) atomicCAS(err, 0, code);
}

struct TileCoord {
    int n, y0, x0;
};
__device__ __forceinline__ TileCoord tile_coord(const TcParams& p, int t) {
    const int tx = t % p.tiles_x, r = t / p.tiles_x;
    return TileCoord{r / p.tiles_y, (r % p.tiles_y) * p.rows, tx * TM};
}

// CK (channels per chunk: 64, 32 or 16) and R (output rows per tile) are
// compile-time so the MMA issue loop unrolls into descriptor additions.
template <int CK, int R>
__global__ void __launch_bounds__(THREADS, 1)
    conv3x3_tc_kernel(const __grid_constant__ CUtensorMap map0, const __grid_constant__ CUtensorMap map1,
                      const TcParams p) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // swizzled operands start on a 1024-byte boundary (the 128-byte swizzle's period)
    uint8_t* smem = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
    uint8_t* sB = smem;
    uint8_t* sA = smem + p.b_stride;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sA + p.stages * p.a_stride);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bars + NBARS);
    volatile int* s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
    float* s_bias = reinterpret_cast<float*>(s_tmem + 4);  // this CTA's n_tile biases
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t full0 = su32(bars), empty0 = su32(bars + MAX_STAGES), tfull0 = su32(bars + 2 * MAX_STAGES),
                   tempty0 = su32(bars + 2 * MAX_STAGES + 2), wbar = su32(bars + 2 * MAX_STAGES + 4),
                   dbar = su32(bars + 2 * MAX_STAGES + 5);
    const int split = blockIdx.x % p.n_split;
    const int cta = blockIdx.x / p.n_split, ncta = gridDim.x / p.n_split;
    const int S = p.stages;

    if (threadIdx.x == 0) {
        for (int s = 0; s < MAX_STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, EPI_WARPS * 32);
        }
        mbar_init(wbar, 1);
        mbar_init(dbar, 1);
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int j = threadIdx.x; j < p.n_tile; j += THREADS) s_bias[j] = p.bias ? p.bias[split * p.n_tile + j] : 0.f;
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(s_tmem)),
                     "r"(p.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;

    if (warp == 0 && lane == 0) {
        // ---- producer: weights once, then (input row, channel chunk) stages ----
        mbar_expect_tx(wbar, p.b_bytes);
        const uint8_t* wsrc = p.wtc + (size_t)split * p.b_bytes;
        for (uint32_t off = 0; off < p.b_bytes; off += 32768u) {
            const uint32_t n = p.b_bytes - off < 32768u ? p.b_bytes - off : 32768u;
            bulk_load(su32(sB) + off, wsrc + off, n, wbar);
        }
        int it = 0;
        bool ok = true;
        for (int t = cta; ok && t < p.pix_tiles; t += ncta) {
            const TileCoord tc = tile_coord(p, t);
            for (int r = 0; ok && r < R + 2; ++r) {
                for (int c = 0; c < p.nchunks; ++c, ++it) {
                    const int s = it % S;
                    if (!mbar_wait(empty0 + 8 * s, ((it / S) & 1) ^ 1, s_abort, p.wait_ns)) {
                        record_error(p.err, s_abort, 2);
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(full0 + 8 * s, p.a_bytes);
                    const int cg = c * p.CK;
                    const bool second = cg >= p.C0;
                    tma_load_4d(su32(sA + s * p.a_stride), second ? &map1 : &map0, second ? cg - p.C0 : cg,
                                tc.x0 - 1, tc.y0 - 1 + r, tc.n, full0 + 8 * s);
                }
            }
        }
        // drain: the last copy into every stage, and the weights, have landed
        for (int i = it - S < 0 ? 0 : it - S; i < it; ++i) mbar_wait(full0 + 8 * (i % S), (i / S) & 1, nullptr, WAIT_NS);
        mbar_wait(wbar, 0, nullptr, WAIT_NS);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t idesc = instr_desc(TM, p.n_tile);
        constexpr uint32_t RB = CK * 2, KS = CK / 16;
        constexpr uint32_t LAYOUT = CK == 64 ? 2u : (CK == 32 ? 4u : 6u);
        const uint32_t b_block = (uint32_t)p.n_tile * RB;  // bytes of one (tap, chunk) block of weights
        const int nkb = p.nchunks;
        bool ok = mbar_wait(wbar, 0, s_abort, p.wait_ns);
        if (!ok) record_error(p.err, s_abort, 1);
        tc_fence_after();
        // descriptors are built once and advanced by adding (byte offset >> 4)
        // to the start-address field (addresses stay below 256 KB)
        const uint64_t b_desc0 = smem_desc(su32(sB), 8 * RB, LAYOUT);
        const uint64_t a_desc0 = smem_desc(su32(sA), 8 * RB, LAYOUT);
        int it = 0, tl = 0;
        for (int t = cta; ok && t < p.pix_tiles; t += ncta, ++tl) {
            const int acc = tl & 1;
            if (!mbar_wait(tempty0 + 8 * acc, ((tl >> 1) & 1) ^ 1, s_abort, p.wait_ns)) {
                record_error(p.err, s_abort, 4);
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t d0 = tmem + (uint32_t)(acc * R * p.n_tile);
            for (int r = 0; ok && r < R + 2; ++r) {
                for (int c = 0; c < nkb; ++c, ++it) {
                    const int s = it % S;
                    if (!mbar_wait(full0 + 8 * s, (it / S) & 1, s_abort, p.wait_ns)) {
                        record_error(p.err, s_abort, 3);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t a_s = a_desc0 + ((uint64_t)(s * p.a_stride) >> 4);
                    const uint64_t b_c = b_desc0 + ((uint64_t)((uint32_t)c * b_block) >> 4);
                    // input row r feeds output row o = r - ky for ky = 0, 1, 2; the
                    // output rows alternate innermost, so consecutive MMAs write
                    // different accumulators. The first MMA into row o's
                    // accumulator is (r = o, ky = 0, c = 0, kx = 0, k step 0).
#pragma unroll
                    for (int kx = 0; kx < 3; ++kx) {
#pragma unroll
                        for (int ks = 0; ks < (int)KS; ++ks) {
                            const uint64_t a = a_s + ((kx * RB + ks * 32) >> 4);
#pragma unroll
                            for (int ky = 0; ky < 3; ++ky) {
                                const int o = r - ky;
                                if (o < 0 || o >= R) continue;
                                const uint64_t b =
                                    b_c + ((uint64_t)((uint32_t)((ky * 3 + kx) * nkb) * b_block + ks * 32) >> 4);
                                mma_f16(d0 + (uint32_t)(o * p.n_tile), a, b, idesc,
                                        (ky | c | kx | ks) != 0 ? 1u : 0u);
                            }
                        }
                    }
                    mma_commit(empty0 + 8 * s);  // the stage is free once these MMAs have read it
                }
            }
            if (ok) mma_commit(tfull0 + 8 * acc);
        }
        // every MMA issued by this thread has completed before tensor memory is freed
        mma_commit(dbar);
        mbar_wait(dbar, 0, nullptr, WAIT_NS);
    } else if (warp >= 2) {
        // ---- epilogue: tensor memory -> bias + activation -> global ----
        const int q = warp & 3;  // this warp's tensor-memory lane quarter
        const int i = q * 32 + lane;
        const int co0 = split * p.n_tile;
        int tl = 0;
        for (int t = cta; t < p.pix_tiles; t += ncta, ++tl) {
            const int acc = tl & 1;
            if (!mbar_wait(tfull0 + 8 * acc, (tl >> 1) & 1, s_abort, p.wait_ns, 256)) {
                record_error(p.err, s_abort, 5);
                break;
            }
            tc_fence_after();
            const TileCoord tc = tile_coord(p, t);
            const int x = tc.x0 + i;
            for (int o = 0; o < R; ++o) {
                const int y = tc.y0 + o;
                for (int j0 = 0; j0 < p.n_tile; j0 += 16) {
                    uint32_t r[16];
                    tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)((acc * R + o) * p.n_tile + j0), r);
                    if (x < p.W && y < p.H) {
                        float v[16];
#pragma unroll
                        for (int k = 0; k < 16; ++k)
                            v[k] = act_fn(__uint_as_float(r[k]) + s_bias[j0 + k], p.act);
                        if (p.out_mode == 0) {
                            __align__(16) __nv_bfloat162 ov[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k) ov[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
                            uint4* dst = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(p.out) +
                                                                  (((size_t)tc.n * p.H + y) * p.W + x) * p.Cout +
                                                                  co0 + j0);
                            dst[0] = reinterpret_cast<const uint4*>(ov)[0];
                            dst[1] = reinterpret_cast<const uint4*>(ov)[1];
                        } else {
                            float4* dst = reinterpret_cast<float4*>(static_cast<float*>(p.out) +
                                                                    (((size_t)tc.n * p.H + y) * p.W + x) * p.Cout +
                                                                    co0 + j0);
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(tempty0 + 8 * acc);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols)
                     : "memory");
    }
}

// ---- weights ----------------------------------------------------------------

// Byte offset of 16-byte chunk `c` of row `r` under the swizzle of rows of
// `rb` bytes (128: chunk ^ (r % 8); 64: chunk ^ (r / 2 % 4); 32: chunk ^ (r / 4 % 2)).
__host__ __device__ inline uint32_t swz(uint32_t r, uint32_t c, uint32_t rb) {
    const uint32_t f = rb == 128 ? (r & 7u) : (rb == 64 ? ((r >> 1) & 3u) : ((r >> 2) & 1u));
    return r * rb + ((c ^ f) << 4);
}

// w [Cout][3][3][Cin] -> wtc[split][tap][chunk][n_tile rows][CK channels], each
// (tap, chunk) block of n_tile rows x CK * 2 bytes swizzled as the operand
// reads it.
__global__ void weights_tc_kernel(const __nv_bfloat16* w, int Cout, int Cin, int n_tile, int CK, __nv_bfloat16* wtc) {
    const long long n = (long long)Cout * 9 * Cin;
    const uint32_t rb = (uint32_t)CK * 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % Cin);
        const int tap = (int)((i / Cin) % 9);
        const int co = (int)(i / (9LL * Cin));
        const int split = co / n_tile, row = co % n_tile;
        const int chunk = ci / CK, k = ci % CK;
        const size_t block = (((size_t)split * 9 + tap) * (Cin / CK) + chunk) * (size_t)n_tile * rb;
        const uint32_t off = swz((uint32_t)row, (uint32_t)(k * 2) >> 4, rb) + ((uint32_t)(k * 2) & 15u);
        wtc[(block + off) / 2] = w[i];
    }
}

unsigned ew_grid(long long n) {
    long long g = (n + 255) / 256;
    return (unsigned)(g < 1 ? 1 : (g > 152LL * 32 ? 152LL * 32 : g));
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(f);
    });
    return fn;
}

// NHWC tensor as 4D {C, W, H, N}; box = CK channels x HALO pixels of one row,
// swizzled by the row width CK * 2 bytes.
bool nhwc_map(CUtensorMap* m, const void* base, int N, int H, int W, int C, int CK) {
    EncodeFn enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[4] = {(cuuint32_t)CK, HALO, 1, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUtensorMapSwizzle sw = CK == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                           : (CK == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int chunk_of(int C0, int C1) { return (C0 % 64 == 0 && C1 % 64 == 0) ? 64 : ((C0 % 32 == 0 && C1 % 32 == 0) ? 32 : 16); }

int status(cudaError_t e) { return e == cudaSuccess ? 0 : 2; }

std::atomic<unsigned long long> g_wait_ns{WAIT_NS};
uint32_t align1024(uint32_t x) { return (x + 1023u) & ~1023u; }

}  // namespace

extern "C" {

int vrc_nn_set_wait_limit(unsigned long long ns) {
    g_wait_ns.store(ns == 0 ? WAIT_NS : ns);
    return 0;
}

int vrc_nn_weights_tc(const void* w, int Cout, int C0, int C1, int n_split, void* wtc, void* stream) {
    const int Cin = C0 + C1;
    if (!w || !wtc || C0 < 16 || C0 % 16 || C1 < 0 || C1 % 16 || n_split < 1 || Cout % n_split ||
        (Cout / n_split) % 16)
        return 1;
    weights_tc_kernel<<<ew_grid((long long)Cout * 9 * Cin), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(w), Cout, Cin, Cout / n_split, chunk_of(C0, C1),
        static_cast<__nv_bfloat16*>(wtc));
    return status(cudaGetLastError());
}

int vrc_nn_conv3x3_tc(const void* in0, int C0, const void* in1, int C1, int N, int H, int W, const void* wtc,
                      const float* bias, int Cout, int n_split, int act, void* out, int out_mode, int* d_err,
                      void* stream) {
    if (!in0 || !wtc || !out || N < 1 || H < 1 || W < 1 || C0 < 16 || C0 % 16 || C1 < 0 || C1 % 16 ||
        (C1 > 0 && !in1) || n_split < 1 || Cout % n_split || act < 0 || act > 2 || out_mode < 0 || out_mode > 1)
        return 1;
    const int n_tile = Cout / n_split;
    if (n_tile % 16 || n_tile > 128) return 4;
    if (((uintptr_t)in0 | (uintptr_t)(in1 ? in1 : in0) | (uintptr_t)wtc | (uintptr_t)out) & 15) return 1;
    const int CK = chunk_of(C0, C1);
    const int Cin = C0 + C1;
    TcParams p{};
    p.N = N;
    p.H = H;
    p.W = W;
    p.C0 = C0;
    p.C1 = C1;
    p.CK = CK;
    p.nchunks = Cin / CK;
    p.n_tile = n_tile;
    p.n_split = n_split;
    p.Cout = Cout;
    p.act = act;
    p.out_mode = out_mode;
    // R output rows per tile: two sets of R accumulators in the 512 columns of
    // tensor memory (one CTA per SM). More rows per tile give each staged
    // input row more MMAs (up to three output rows read it), which covers the
    // TMA round trip of the next stage when the weights leave room for few
    // stages (64 -> 128: 147 KB of weights, 3 stages)
    int R = 256 / n_tile;
    if (R > MAX_ROWS) R = MAX_ROWS;
    if (R < 1) R = 1;
    p.rows = R;
    p.tiles_x = (W + TM - 1) / TM;
    p.tiles_y = (H + R - 1) / R;
    const long long pix_tiles = (long long)N * p.tiles_y * p.tiles_x;
    if (pix_tiles > (1LL << 30)) return 1;
    p.pix_tiles = (int)pix_tiles;
    uint32_t cols = 32;
    while (cols < 2u * (uint32_t)(R * n_tile)) cols <<= 1;
    p.tmem_cols = cols;
    p.row_bytes = (uint32_t)CK * 2;
    p.layout = CK == 64 ? 2u : (CK == 32 ? 4u : 6u);
    p.a_bytes = (uint32_t)HALO * p.row_bytes;
    p.a_stride = align1024(p.a_bytes);
    p.b_bytes = 9u * (uint32_t)Cin * (uint32_t)n_tile * 2u;
    p.b_stride = align1024(p.b_bytes);
    const size_t fixed = 1024 + (size_t)p.b_stride + NBARS * 8 + 16 + 128 * sizeof(float);
    if (fixed + 2 * (size_t)p.a_stride > SMEM_BUDGET) return 4;
    long long stages = (long long)((SMEM_BUDGET - fixed) / p.a_stride);
    if (stages > MAX_STAGES) stages = MAX_STAGES;
    p.stages = (int)stages;
    p.bias = bias;
    p.wtc = static_cast<const uint8_t*>(wtc);
    p.out = out;
    p.err = d_err;
    p.wait_ns = g_wait_ns.load();
    const size_t smem = fixed + (size_t)p.stages * p.a_stride;
    CUtensorMap m0, m1;
    if (!nhwc_map(&m0, in0, N, H, W, C0, CK)) return 2;
    if (!nhwc_map(&m1, C1 > 0 ? in1 : in0, N, H, W, C1 > 0 ? C1 : C0, CK)) return 2;
    using Kernel = void (*)(const CUtensorMap, const CUtensorMap, const TcParams);
    Kernel k = nullptr;
#define VRC_TC_PICK(ck, r) \
    if (CK == ck && R == r) k = conv3x3_tc_kernel<ck, r>;
    VRC_TC_PICK(64, 1) VRC_TC_PICK(64, 2) VRC_TC_PICK(64, 4)
    VRC_TC_PICK(32, 1) VRC_TC_PICK(32, 2) VRC_TC_PICK(32, 4)
    VRC_TC_PICK(16, 1) VRC_TC_PICK(16, 2) VRC_TC_PICK(16, 4)
#undef VRC_TC_PICK
    if (!k) return 4;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return 2;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return 2;
    // one CTA per SM (the shared-memory budget); ctas are split evenly between channel slices
    long long per_split = sms / n_split;
    if (per_split < 1) per_split = 1;
    if (per_split > pix_tiles) per_split = pix_tiles;
    k<<<(unsigned)(per_split * n_split), THREADS, smem, static_cast<cudaStream_t>(stream)>>>(m0, m1, p);
    return status(cudaGetLastError());
}

}  // extern "C"
