// Plain FP32 SIMT GEMM: the Hankel products of the reference-ordered linear step.
//
// LinearOperator.half_linear (operators.py:48, :53) multiplies the real QDHT
// matrix Y (Nr x Nr) into the complex field (Nr x Nt); cp.dot promotes Y to
// complex, so the reference runs a ZGEMM with 4x the useful flops.  Here the
// field's interleaved (re, im) columns are treated as 2*Nt real columns:
// C[M x N] = A[M x K] * B[K x N] with M = K = Nr, N = 2 Nt, all row-major
// FP32, and an optional per-row scale in the epilogue (the radial absorber
// mask_r, integrator.py:149).  This is the "plain FP32" form; the split-BF16
// tensor-core form replaces it on the fast path.
//
// 128x128 CTA tile, 8-deep k slices double-buffered through shared memory,
// 256 threads each accumulating an 8x8 register block (two 4-wide strips per
// dimension so the shared-memory fragment reads are conflict-free float4s).
#include "nlse_internal.cuh"

#define GB_M 128
#define GB_N 128
#define GB_K 8

__global__ void __launch_bounds__(256)
k_gemm_f32(const float *__restrict__ A, const float *__restrict__ B, float *__restrict__ C, int M, int N,
           int K, const float *__restrict__ row_scale) {
    __shared__ __align__(16) float As[2][GB_K][GB_M];
    __shared__ __align__(16) float Bs[2][GB_K][GB_N];
    const int tid = threadIdx.x;
    const int bm = blockIdx.y * GB_M, bn = blockIdx.x * GB_N;
    const int tx = tid & 15, ty = tid >> 4;
    // global->smem load assignment: A: row = tid/2, k = (tid&1)*4 .. +3 ; B: k = tid/32, n = (tid&31)*4 .. +3
    const int la_m = tid >> 1, la_k = (tid & 1) * 4;
    const int lb_k = tid >> 5, lb_n = (tid & 31) * 4;

    float ra[4], rb[4];
    auto load_tile = [&](int k0) {
        const int gm = bm + la_m;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int gk = k0 + la_k + q;
            ra[q] = (gm < M && gk < K) ? __ldg(&A[(size_t)gm * K + gk]) : 0.0f;
        }
        const int gk = k0 + lb_k;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int gn = bn + lb_n + q;
            rb[q] = (gk < K && gn < N) ? __ldg(&B[(size_t)gk * N + gn]) : 0.0f;
        }
    };
    auto store_tile = [&](int buf) {
#pragma unroll
        for (int q = 0; q < 4; ++q) As[buf][la_k + q][la_m] = ra[q];
        *reinterpret_cast<float4 *>(&Bs[buf][lb_k][lb_n]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    load_tile(0);
    store_tile(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = 0; k0 < K; k0 += GB_K) {
        const bool more = k0 + GB_K < K;
        if (more) load_tile(k0 + GB_K);
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
            float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][64 + ty * 4]);
            float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
            float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][64 + tx * 4]);
            float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) {
            store_tile(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int gm = bm + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (gm >= M) continue;
        const float s = row_scale ? __ldg(&row_scale[gm]) : 1.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int gn = bn + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (gn < N) C[(size_t)gm * N + gn] = acc[i][j] * s;
        }
    }
}

cudaError_t launch_gemm_f32(const float *A, const float *B, float *C, int M, int N, int K,
                            const float *row_scale, cudaStream_t stream) {
    dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M);
    k_gemm_f32<<<grid, 256, 0, stream>>>(A, B, C, M, N, K, row_scale);
    return cudaGetLastError();
}
