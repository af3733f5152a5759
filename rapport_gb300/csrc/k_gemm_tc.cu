// Split-BF16 tcgen05 GEMM for the merged linear operator, and its builder.
//
// The reference's linear half step (operators.py:47-53) is
//     iRk Y ifft_t( e^{i phi} mask fft_t( Rk Y u ) ),   phi = dk(W) dz/2 - rho_m^2 dz/(4 k0)
// with two real Nr x Nr QDHT products around an FFT pair.  Y acts on r and the
// FFT on t, so they commute, and the radial phase diag(P_r) is diagonal in the
// Hankel basis: the half step is
//     F^-1[ P_t . (M F[u]) ],   M = Y diag(P_r) Y = I + E     (Rk iRk = 1).
// M is one complex Nr x Nr matrix per dz.  In the Omega domain the field is
// stored planar, w' = [Re w; Im w] (2 Nr x Nt), and
//     E' = [[Re E, -Im E], [Im E, Re E]]      (2 Nr x 2 Nr, real)
// so E' w' is ONE real GEMM of M = K = 2 Nr, N = Nt (8 Nr^2 Nt flops, the same
// as the reference's two complex-promoted products counted as real work).
// The identity part of M is added exactly in FP32 by the row kernel that
// consumes the product; only E -- |E| <= 0.15, typically |E w| ~ 1e-3 |w| --
// goes through the tensor cores.
//
// Precision: E' is split into three BF16 terms (h + m + l, ~24 bits) and the
// field into two (h + l, ~16 bits); the MMAs Eh.wh + Eh.wl + Em.wh + El.wh
// accumulate in FP32 in TMEM (A_TERMS = 3; A_TERMS = 2 drops El.wh: the plain
// hi/lo 3-MMA scheme).  E's own rounding is systematic and would accumulate
// over thousands of steps; carrying it in three terms removes that drift.
//
// Kernel: persistent, 128 x 256 output tiles, one CTA per SM; warp 0 = TMA
// producer, warp 1 = TMEM allocator + MMA issuer (one elected thread), warps
// 2-5 = epilogue (tcgen05.ld of their 32-lane TMEM quadrant, FP32 rows to
// global) on a double-buffered TMEM accumulator.  Operands are staged by TMA
// (128- or 64-byte swizzle) into an mbarrier ring of 2-4 stages: A tiles
// K-major (box BK x 128), B tiles MN-major (4 boxes of 64 x BK).
// Every wait is bounded by %globaltimer; on timeout the kernel raises an
// error word, drains what it issued, frees TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>

#include "nlse_internal.cuh"

#define TC_BM 128
#define TC_BN 256
#define TC_THREADS 192
#define TC_WAIT_NS 2000000000ull

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity to complete; false once limit_ns
// (2 s for the product's waits) have passed.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns = TC_WAIT_NS) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 1;; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255u) == 0 && global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor (tcgen05): start, leading/stride byte
// offsets (>> 4), version 1, swizzle mode (2 = 128-byte, 4 = 64-byte).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo, uint32_t swz) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)swz << 61;
    return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace

// Instruction descriptor, kind::f16: FP32 accumulate, BF16 (F16 = false) or
// FP16 (F16 = true) A and B, A K-major, B MN-major, N = 256, M = 128.
template <bool F16>
constexpr uint32_t idesc_f16() {
    return (1u << 4) | (F16 ? 0u : (1u << 7) | (1u << 10)) | (1u << 16) | ((uint32_t)(TC_BN >> 3) << 17) |
           ((uint32_t)(TC_BM >> 4) << 24);
}

// Where the tiles of a launch come from: one product D[M x N] = A B tiled
// row-major (tiles == NULL), or a table of (pulse, m0, n0) over the pulses of
// a batch, each with its own tensor maps (global memory) and sizes.
struct TileSource {
    const CUtensorMap *tmA, *tmB;  // single product
    float *D;
    int M, N, K;
    int kdiag;                     // single product: block-diagonal operator
    const GemmTile *tiles;         // grouped: tile table, maps, pulses
    const CUtensorMap *maps;
    const BatchPulse *P;
    int map_off;                   // 0: the k-64 maps of a pulse, 2: the k-32 maps
};

struct TileJob {
    const CUtensorMap *tmA, *tmB;
    float *D;
    int M, N, K, m0, n0;
    int k0, kn;  // the K range the tile contracts: all of K, or with a block-diagonal
                 // operator (M = K = two blocks) the range of the tile's row block
};

__device__ __forceinline__ TileJob tile_job(const TileSource &src, int t) {
    TileJob j;
    if (src.tiles) {
        const GemmTile g = src.tiles[t];
        const BatchPulse &q = src.P[g.pulse];
        j.tmA = src.maps + 4 * g.pulse + src.map_off;
        j.tmB = j.tmA + 1;
        j.D = q.D;
        j.M = q.M;
        j.N = q.N;
        j.K = q.K;
        j.m0 = g.m0;
        j.n0 = g.n0;
        j.k0 = q.kdiag;  // flag, resolved below
    } else {
        const int nt = (src.N + TC_BN - 1) / TC_BN;
        j.tmA = src.tmA;
        j.tmB = src.tmB;
        j.D = src.D;
        j.M = src.M;
        j.N = src.N;
        j.K = src.K;
        j.m0 = (t / nt) * TC_BM;
        j.n0 = (t % nt) * TC_BN;
        j.k0 = src.kdiag;
    }
    if (j.k0) {
        j.kn = j.K / 2;
        j.k0 = j.m0 >= j.M / 2 ? j.kn : 0;
    } else {
        j.kn = j.K;
    }
    return j;
}

// Persistent warp-specialised product: CTA b computes tiles b, b + G, b + 2G,
// ... (G = gridDim.x, at most one CTA per SM).  The TMA producer runs the
// stage ring across tile boundaries, and the accumulator is double-buffered
// in TMEM (2 x 256 columns): while the epilogue warps drain tile i from one
// buffer, the MMA issuer already accumulates tile i + 1 into the other, so the
// tensor pipe does not wait for the epilogue, the pipeline fill or the CTA
// set-up of the next tile.  Each tile's MMA sequence is exactly that of a
// single-tile CTA (same k order, first MMA without accumulate).
//   warp 0: TMA producer; warp 1: TMEM allocator + MMA issuer; warps 2-5:
//   epilogue (each its 32-lane TMEM quadrant).
// Every wait is bounded by %globaltimer; on timeout the CTA raises an error
// bit, stops issuing, waits (bounded) for the copies and MMAs it issued,
// frees TMEM and returns.
template <int A_TERMS, int TC_BK, int TC_STAGES, bool F16>
__device__ __forceinline__ void gemm_persistent(const TileSource &src, int ntiles, int *__restrict__ err) {
    constexpr uint32_t kIdesc = idesc_f16<F16>();
    constexpr uint32_t A_BYTES = TC_BM * TC_BK * 2;  // one term
    constexpr uint32_t B_BYTES = TC_BK * TC_BN * 2;  // one term
    constexpr uint32_t B_BOX = 64 * TC_BK * 2;       // one 64-column box
    constexpr uint32_t STAGE = A_TERMS * A_BYTES + 2 * B_BYTES;
    constexpr uint32_t A_SWZ = TC_BK == 64 ? 2u : 4u;
    constexpr uint32_t A_SBO = TC_BK * 2 * 8;        // 8 rows of one swizzle atom
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full_bar[TC_STAGES], empty_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag, issued;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], 4);  // one arrival per epilogue warp
        }
        mbar_init(&done_bar, 1);
        abort_flag = 0;
        issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base)),
                     "r"(2 * TC_BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        // ------------------------------------------------ TMA producer
        int g = 0;  // stage sequence number across tiles
        for (int t = blockIdx.x; t < ntiles && !*(volatile int *)&abort_flag; t += gridDim.x) {
            const TileJob j = tile_job(src, t);
            const int KB = j.kn / TC_BK;
            for (int kb = 0; kb < KB; ++kb, ++g) {
                const int s = g % TC_STAGES;
                const uint32_t ph = (uint32_t)(g / TC_STAGES) & 1u;
                if (!mbar_wait(&empty_bar[s], ph ^ 1u) || *(volatile int *)&abort_flag) {
                    atomicOr(err, 1);
                    abort_flag = 1;
                    break;
                }
                uint8_t *st = smem + (size_t)s * STAGE;
                mbar_expect_tx(&full_bar[s], STAGE);
#pragma unroll
                for (int a = 0; a < A_TERMS; ++a)
                    tma_load_2d(st + a * A_BYTES, j.tmA, &full_bar[s], j.k0 + kb * TC_BK, a * j.M + j.m0);
#pragma unroll
                for (int b = 0; b < 2; ++b)
#pragma unroll
                    for (int c = 0; c < TC_BN / 64; ++c)
                        tma_load_2d(st + A_TERMS * A_BYTES + b * B_BYTES + c * B_BOX, j.tmB, &full_bar[s],
                                    j.n0 + 64 * c, b * j.K + j.k0 + kb * TC_BK);
                issued = g + 1;
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ------------------------------------------------ MMA issuer
        // term pairs (a, b): Eh.wh, Eh.wl, Em.wh [, El.wh]  (FP16: Eh.wh, Eh.wl, El.wh)
        const int pa[4] = {0, 0, 1, 2}, pb[4] = {0, 1, 0, 0};
        constexpr int NPAIR = A_TERMS == 3 ? 4 : 3;
        int g = 0, i = 0;
        for (int t = blockIdx.x; t < ntiles && !*(volatile int *)&abort_flag; t += gridDim.x, ++i) {
            const int acc = i & 1;
            const uint32_t d_tmem = tmem + (uint32_t)(acc * TC_BN);
            // the epilogue has drained this buffer (tile i - 2)
            if (!mbar_wait(&acc_empty[acc], (((uint32_t)i >> 1) & 1u) ^ 1u)) {
                atomicOr(err, 2);
                abort_flag = 1;
                break;
            }
            tc_fence_after();
            const int KB = tile_job(src, t).kn / TC_BK;
            bool ok = true;
            for (int kb = 0; kb < KB; ++kb, ++g) {
                const int s = g % TC_STAGES;
                const uint32_t ph = (uint32_t)(g / TC_STAGES) & 1u;
                if (!mbar_wait(&full_bar[s], ph) || *(volatile int *)&abort_flag) {
                    atomicOr(err, 2);
                    abort_flag = 1;
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = smem_u32(smem + (size_t)s * STAGE);
                const uint32_t b0 = a0 + A_TERMS * A_BYTES;
#pragma unroll
                for (int kk = 0; kk < TC_BK / 16; ++kk) {
#pragma unroll
                    for (int p = 0; p < NPAIR; ++p) {
                        const uint64_t ad = smem_desc(a0 + pa[p] * A_BYTES + kk * 32, 16, A_SBO, A_SWZ);
                        const uint64_t bd = smem_desc(b0 + pb[p] * B_BYTES + kk * 2048, B_BOX, 1024, 2u);
                        umma_bf16(d_tmem, ad, bd, kIdesc, (kb | kk | p) != 0);
                    }
                }
                umma_commit(&empty_bar[s]);
            }
            if (!ok) break;
            umma_commit(&acc_full[acc]);
        }
        umma_commit(&done_bar);  // always: teardown waits for every MMA issued here
    } else if (warp >= 2) {
        // ------------------------------------------------ epilogue
        const int q = warp & 3;
        int i = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
            const int acc = i & 1;
            if (!mbar_wait(&acc_full[acc], ((uint32_t)i >> 1) & 1u)) {
                atomicOr(err, 4);
                abort_flag = 1;
                break;
            }
            if (*(volatile int *)&abort_flag) break;
            tc_fence_after();
            const TileJob j = tile_job(src, t);
            float *row = j.D + (size_t)(j.m0 + q * 32 + lane) * j.N + j.n0;
            const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * TC_BN);
            // columns of the tile inside D (N < 256: one partial tile; N is a multiple of 16)
            const int ncol = min(TC_BN, j.N - j.n0);
#pragma unroll 1
            for (int c = 0; c < TC_BN / 32; ++c) {
                if (c * 32 >= ncol) break;  // warp-uniform: tcgen05.ld stays converged
                uint32_t r[32];
                tmem_ld32(tq + (uint32_t)(c * 32), r);
                float4 *dst = reinterpret_cast<float4 *>(row + c * 32);
#pragma unroll
                for (int v = 0; v < 8; ++v)
                    if (c * 32 + 4 * v < ncol)
                        dst[v] = make_float4(__uint_as_float(r[4 * v]), __uint_as_float(r[4 * v + 1]),
                                             __uint_as_float(r[4 * v + 2]), __uint_as_float(r[4 * v + 3]));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[acc]))
                                        : "memory");
        }
    }
    tc_fence_before();
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) {
        // drain: the last loads this CTA issued must land before it exits
        for (int g = issued - TC_STAGES; g < issued; ++g)
            if (g >= 0) mbar_wait(&full_bar[g % TC_STAGES], (uint32_t)(g / TC_STAGES) & 1u);
    }
    if (warp == 1) {
        if (lane == 0) mbar_wait(&done_bar, 0);  // every MMA done before TMEM is released
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_BN));
    }
}

template <int A_TERMS, int BK, int ST, bool F16>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
          float *__restrict__ D, int M, int N, int K, int kdiag, int *__restrict__ err) {
    TileSource src{&tmA, &tmB, D, M, N, K, kdiag, nullptr, nullptr, nullptr, 0};
    gemm_persistent<A_TERMS, BK, ST, F16>(src, (M / TC_BM) * ((N + TC_BN - 1) / TC_BN), err);
}

// Grouped product over many pulses: the tiles of tiles[0 .. ntiles) of pulse
// tiles[t].pulse, whose tensor maps are maps[4 p ..] (global memory, written
// by the host before the launch): [4p] A (box 64), [4p+1] B (box 64),
// [4p+2] A (box 32), [4p+3] B (box 32).
template <int A_TERMS, int BK, int ST, bool F16>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_gemm_tc_grouped(const CUtensorMap *__restrict__ maps, const BatchPulse *__restrict__ P,
                  const GemmTile *__restrict__ tiles, int ntiles, int *__restrict__ err) {
    TileSource src{nullptr, nullptr, nullptr, 0, 0, 0, 0, tiles, maps, P, BK == 32 ? 2 : 0};
    gemm_persistent<A_TERMS, BK, ST, F16>(src, ntiles, err);
}

// One CTA per SM at most (the stage ring and the 512 TMEM columns fill it).
static int tc_grid(int ntiles) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
            sms = 1;
    }
    return ntiles < sms ? ntiles : sms;
}

// Dynamic shared memory of a pipeline variant; never less than 120 KB, so two
// CTAs of the product can not share an SM (each allocates all 512 TMEM columns).
static size_t tc_smem_bytes(int a_terms, int bk, int stages) {
    const size_t need = (size_t)stages * (a_terms * TC_BM * bk * 2 + 2 * bk * TC_BN * 2) + 1024;
    return need < 120 * 1024 ? 120 * 1024 : need;
}

// variant: 0 = (BK 64, 2 stages), 1 = (BK 32, 4 stages), 2 = (BK 32, 3 stages),
// 3 = (BK 32, 2 stages).  2 and 3 leave shared memory for a row-kernel CTA
// on the same SM (169 KB / 116 KB of the 228 KB).
#define TC_DISPATCH_AT(AT_, F16_, variant, ...)                                                   \
    if (variant == 0) { constexpr int AT = AT_, BK = 64, ST = 2; constexpr bool F16 = F16_; __VA_ARGS__; }      \
    else if (variant == 1) { constexpr int AT = AT_, BK = 32, ST = 4; constexpr bool F16 = F16_; __VA_ARGS__; } \
    else if (variant == 2) { constexpr int AT = AT_, BK = 32, ST = 3; constexpr bool F16 = F16_; __VA_ARGS__; } \
    else { constexpr int AT = AT_, BK = 32, ST = 2; constexpr bool F16 = F16_; __VA_ARGS__; }
// BF16: 3 or 2 operator terms; FP16: 2 operator terms (3 MMAs), or 3 (4 MMAs: the
// space-time-focusing operator Y, whose rounding is applied twice per half step)
#define TC_DISPATCH(a_terms, f16, variant, ...)                                                  \
    if (f16 && a_terms == 3) { TC_DISPATCH_AT(3, true, variant, __VA_ARGS__) }                   \
    else if (f16) { TC_DISPATCH_AT(2, true, variant, __VA_ARGS__) }                              \
    else if (a_terms == 3) { TC_DISPATCH_AT(3, false, variant, __VA_ARGS__) }                    \
    else { TC_DISPATCH_AT(2, false, variant, __VA_ARGS__) }

cudaError_t launch_gemm_tc_grouped(const CUtensorMap *maps, const BatchPulse *P, const GemmTile *tiles, int ntiles,
                                   int a_terms, int variant, int f16, int *err, cudaStream_t stream) {
    TC_DISPATCH(a_terms, f16, variant, {
        const size_t smem = tc_smem_bytes(AT, BK, ST);
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc_grouped<AT, BK, ST, F16>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_tc_grouped<AT, BK, ST, F16>
            <<<tc_grid(ntiles), TC_THREADS, smem, stream>>>(maps, P, tiles, ntiles, err);
    })
    return cudaGetLastError();
}

cudaError_t launch_gemm_tc(const CUtensorMap *tmA, const CUtensorMap *tmB, float *D, int M, int N, int K,
                           int a_terms, int variant, int f16, int kdiag, int *err, cudaStream_t stream) {
    if (M % TC_BM || N % 16 || K % 64 || (kdiag && (M != K || (K / 2) % 64 || (M / 2) % TC_BM)))
        return cudaErrorInvalidValue;
    const int grid = tc_grid((M / TC_BM) * ((N + TC_BN - 1) / TC_BN));
    TC_DISPATCH(a_terms, f16, variant, {
        const size_t smem = tc_smem_bytes(AT, BK, ST);
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<AT, BK, ST, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_tc<AT, BK, ST, F16><<<grid, TC_THREADS, smem, stream>>>(*tmA, *tmB, D, M, N, K, kdiag, err);
    })
    return cudaGetLastError();
}

// ------------------------------------------------------------------ failure-path probe
// The product's bounded wait and its error reporting, exercised on purpose:
// one thread waits on an mbarrier that nothing arrives on, with the caller's
// (short) limit instead of the product's 2 s, then raises the status bit the
// product raises on a timeout (bit 3: the probe) and returns.  The barrier
// lives in this CTA's shared memory and no copy or MMA is issued, so the
// kernel leaves nothing in flight.
__global__ void k_wait_probe(int *__restrict__ err, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!mbar_wait(&bar, 0, limit_ns)) atomicOr(err, 8);
}

cudaError_t launch_wait_probe(int *err, unsigned long long limit_ns, cudaStream_t stream) {
    k_wait_probe<<<1, 32, 0, stream>>>(err, limit_ns);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ operator builder (FP64)
// Er + i Ei = Y diag(e^{i theta}) Y - I,  theta_k = -rho_k^2 dz / (4 k0).
// 32 x 32 output tiles, 16-deep k slices through shared memory; each thread
// accumulates a 2 x 2 block of (Er, Ei) pairs.  Runs once per dz.
__global__ void __launch_bounds__(256)
k_build_E(const double *__restrict__ Y, const double *__restrict__ rho, int Nr, double dz, double komega,
          double *__restrict__ Er, double *__restrict__ Ei) {
    __shared__ double As[32][17], Bc[16][33], Bs[16][33];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int row0 = blockIdx.y * 32, col0 = blockIdx.x * 32;
    double ar[2][2] = {{0, 0}, {0, 0}}, ai[2][2] = {{0, 0}, {0, 0}};
    for (int k0 = 0; k0 < Nr; k0 += 16) {
        for (int i = threadIdx.x; i < 32 * 16; i += 256) {
            int r = i / 16, k = i % 16;
            int gr = row0 + r, gk = k0 + k;
            As[r][k] = (gr < Nr && gk < Nr) ? Y[(size_t)gr * Nr + gk] : 0.0;
        }
        for (int i = threadIdx.x; i < 16 * 32; i += 256) {
            int k = i / 32, cc = i % 32;
            int gk = k0 + k, gc = col0 + cc;
            double y = (gk < Nr && gc < Nr) ? Y[(size_t)gk * Nr + gc] : 0.0;
            double s = 0.0, c = 0.0;
            if (gk < Nr) {
                double rr = rho[gk];
                sincos(-rr * rr * dz / (4.0 * komega), &s, &c);
            }
            Bc[k][cc] = c * y;
            Bs[k][cc] = s * y;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                double a = As[ty * 2 + i][k];
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    ar[i][j] = fma(a, Bc[k][tx * 2 + j], ar[i][j]);
                    ai[i][j] = fma(a, Bs[k][tx * 2 + j], ai[i][j]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            int r = row0 + ty * 2 + i, cc = col0 + tx * 2 + j;
            if (r < Nr && cc < Nr) {
                Er[(size_t)r * Nr + cc] = ar[i][j] - (r == cc ? 1.0 : 0.0);
                Ei[(size_t)r * Nr + cc] = ai[i][j];
            }
        }
}

// Entry (m, k) of E' = [[Er, -Ei], [Ei, Er]] in the padded layout: blocks of
// Nrp rows / columns, of which the first Nr hold E and the rest are zero.
__device__ __forceinline__ double e_prime(const double *__restrict__ Er, const double *__restrict__ Ei, int Nr,
                                          int Nrp, size_t m, size_t k) {
    const size_t mr = m % Nrp, kr = k % Nrp;
    if (mr >= (size_t)Nr || kr >= (size_t)Nr) return 0.0;
    const bool mi = m >= (size_t)Nrp, ki = k >= (size_t)Nrp;
    return (mi == ki) ? Er[mr * Nr + kr] : (mi ? Ei[mr * Nr + kr] : -Ei[mr * Nr + kr]);
}

// E' split into a_terms BF16 terms, stacked as A[t][2Nrp][2Nrp] (term-major):
// h = bf16(v), m = bf16(v - h), l = bf16(v - h - m).
__global__ void k_split_E(const double *__restrict__ Er, const double *__restrict__ Ei, int Nr, int Nrp, int a_terms,
                          __nv_bfloat16 *__restrict__ A) {
    const size_t K2 = 2 * (size_t)Nrp;
    const size_t total = K2 * K2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const double v = e_prime(Er, Ei, Nr, Nrp, i / K2, i % K2);
        double rem = v;
        for (int t = 0; t < a_terms; ++t) {
            __nv_bfloat16 b = __double2bfloat16(rem);
            A[(size_t)t * total + i] = b;
            rem -= (double)__bfloat162float(b);
        }
    }
}

// max |E| (float bits; every entry of Er and Ei) into scale[NLSE_SC_EMAX].
__global__ void k_absmax_E(const double *__restrict__ Er, const double *__restrict__ Ei, size_t n,
                           int *__restrict__ scale) {
    float mx = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        mx = fmaxf(mx, (float)fmax(fabs(Er[i]), fabs(Ei[i])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&scale[NLSE_SC_EMAX], __float_as_int(mx));
}

// E' 2^sa as two FP16 terms (h + l, ~22 bits), sa = 14 - e with max |E| < 2^e:
// the largest entry lands in [2^13, 2^14), far from FP16's 65504, and entries
// down to 2^-11 of it keep both terms normal.  sa goes to scale[NLSE_SC_SA].
__global__ void k_split_E16(const double *__restrict__ Er, const double *__restrict__ Ei, int Nr, int Nrp,
                            __half *__restrict__ A, int *__restrict__ scale) {
    const float emax = __int_as_float(scale[NLSE_SC_EMAX]);
    int e = 0;
    if (emax > 0.0f && isfinite(emax)) frexpf(emax, &e);
    const int sa = min(max(14 - e, -100), 100);
    if (blockIdx.x == 0 && threadIdx.x == 0) scale[NLSE_SC_SA] = sa;
    const double sc = ldexp(1.0, sa);
    const size_t K2 = 2 * (size_t)Nrp;
    const size_t total = K2 * K2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const double v = e_prime(Er, Ei, Nr, Nrp, i / K2, i % K2) * sc;
        const __half h = __double2half(v);
        A[i] = h;
        A[total + i] = __double2half(v - (double)__half2float(h));
    }
}

cudaError_t launch_build_operator(const double *Y64, const double *rho, int Nr, int Nrp, double dz, double komega,
                                  double *Er, double *Ei, int a_terms, __nv_bfloat16 *A, int f16, int *scale,
                                  cudaStream_t stream) {
    dim3 grid((Nr + 31) / 32, (Nr + 31) / 32);
    k_build_E<<<grid, 256, 0, stream>>>(Y64, rho, Nr, dz, komega, Er, Ei);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (!f16) {
        k_split_E<<<1024, 256, 0, stream>>>(Er, Ei, Nr, Nrp, a_terms, A);
        return cudaGetLastError();
    }
    e = cudaMemsetAsync(scale + NLSE_SC_EMAX, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    k_absmax_E<<<304, 256, 0, stream>>>(Er, Ei, (size_t)Nr * Nr, scale);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_split_E16<<<1024, 256, 0, stream>>>(Er, Ei, Nr, Nrp, reinterpret_cast<__half *>(A), scale);
    return cudaGetLastError();
}
