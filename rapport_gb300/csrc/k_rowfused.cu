// Fused row kernels of the split-BF16 path (one CTA per radius r).
//
// Between z-steps the field is kept in the Omega domain, w = F[u], stored
// planar (row r = Re, row Nr + r = Im) in FP32 plus its BF16 hi/lo terms --
// the B operand of the tensor-core product E' w'.  One z-step of
// Integrator.propagate (update_plasma + step, integrator.py:138-158) becomes
//
//   G1      D  = E' w                                (k_gemm_tc)
//   row_nl  x  = P_t (w + D); u = F^-1[x]; u <- NL(u, rho); y = F[u]
//   G2      D  = E' y                                (k_gemm_tc)
//   row_nx  w' = mask_r P_t (y + D); u' = F^-1[w']; rho <- march(|u'|^2)
//
// where P_t = e^{i dk dz/2} spec_mask, the identity part of M = I + E is
// added here exactly in FP32, and row_nx's march is the NEXT iteration's
// update_plasma (the entry kernel does the first one).  Each row kernel reads
// and writes its row once (HBM) and does the FFTs, the nonlinear block and the
// scan in shared memory.
#include <cuda_bf16.h>

#include "nl_impl.cuh"
#include "scan_impl.cuh"


// FP32 planar rows + BF16 hi/lo terms of one complex row held in smem.
__device__ __forceinline__ void store_state_row(const float2 *s, int r, const RowFusedArgs &a, float *F32,
                                                __nv_bfloat16 *Fb) {
    const size_t Nt = a.Nt, rows = 2 * (size_t)a.Nr;
    float *re = F32 + (size_t)r * Nt, *im = F32 + ((size_t)a.Nr + r) * Nt;
    __nv_bfloat16 *hre = Fb + (size_t)r * Nt, *him = Fb + ((size_t)a.Nr + r) * Nt;
    __nv_bfloat16 *lre = hre + rows * Nt, *lim = him + rows * Nt;
    for (int t = threadIdx.x; t < a.Nt; t += blockDim.x) {
        float2 v = s[t];
        re[t] = v.x;
        im[t] = v.y;
        __nv_bfloat16 hx = __float2bfloat16_rn(v.x), hy = __float2bfloat16_rn(v.y);
        hre[t] = hx;
        him[t] = hy;
        lre[t] = __float2bfloat16_rn(v.x - __bfloat162float(hx));
        lim[t] = __float2bfloat16_rn(v.y - __bfloat162float(hy));
    }
}

// s[t] = scale * P_t[t] * ((F32 + D) row r as complex)
__device__ __forceinline__ void load_mw_row(float2 *s, int r, const RowFusedArgs &a, const float *F32,
                                            const float *D, float scale) {
    const size_t Nt = a.Nt;
    const float *fr = F32 + (size_t)r * Nt, *fi = F32 + ((size_t)a.Nr + r) * Nt;
    const float *dr = D + (size_t)r * Nt, *di = D + ((size_t)a.Nr + r) * Nt;
    for (int t = threadIdx.x; t < a.Nt; t += blockDim.x) {
        float2 z = make_float2(fr[t] + dr[t], fi[t] + di[t]);
        s[t] = c_scale(c_mul(z, __ldg(&a.Pt[t])), scale);
    }
}

// Entry: physical u (interleaved) -> w = F[u] (state); optionally rho = march(|u|^2).
__global__ void __launch_bounds__(NLSE_ROW_THREADS)
k_row_entry(RowFusedArgs a, const float2 *__restrict__ u, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb,
            float *__restrict__ rho, int do_scan) {
    extern __shared__ float2 sm2[];
    const int r = blockIdx.x, Nt = a.Nt;
    float2 *b0 = sm2, *b1 = sm2 + Nt;
    const float2 *g = u + (size_t)r * Nt;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) b0[t] = g[t];
    __syncthreads();
    float2 *R = fft_row<false>(b0, b1, Nt, a.logNt, a.tw);
    store_state_row(R, r, a, F32, Fb);
    if (!do_scan) return;
    __syncthreads();
    float *sI = (float *)(R == b0 ? b1 : b0), *sW = sI + Nt;
    float *sx = (float *)R, *sJ = sx + Nt, *sB = (float *)(sm2 + 2 * Nt);
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        float2 v = g[t];
        sI[t] = fmaf(v.x, v.x, v.y * v.y) * a.sc.invE2;
    }
    __syncthreads();
    scan_row(sI, sW, sx, sJ, sB, Nt, a.sc, a.lut, 0.0f, a.stats);
    float *gr = rho + (size_t)r * Nt;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) gr[t] = sx[t];
}

// First half step's spectral end + the nonlinear block + forward FFT.
__global__ void __launch_bounds__(NLSE_ROW_THREADS)
k_row_nl(RowFusedArgs a, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
         const float *__restrict__ rho) {
    extern __shared__ float2 sm2[];
    const int r = blockIdx.x, Nt = a.Nt;
    float2 *b0 = sm2, *b1 = sm2 + Nt;
    load_mw_row(b0, r, a, F32, D, 1.0f / (float)Nt);
    __syncthreads();
    float2 *R = fft_row<true>(b0, b1, Nt, a.logNt, a.tw);
    const float *gr = rho + (size_t)r * Nt;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) R[t] = nl_point(R[t], gr[t], a.dz, a.nl, a.pchip);
    __syncthreads();
    float2 *O = R == b0 ? b1 : b0;
    float2 *Y = fft_row<false>(R, O, Nt, a.logNt, a.tw);
    store_state_row(Y, r, a, F32, Fb);
}

// Second half step's spectral end + mask_r: the next state w', and optionally
// the physical field (u_out) and the next carrier march (rho).
__global__ void __launch_bounds__(NLSE_ROW_THREADS)
k_row_next(RowFusedArgs a, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
           float *__restrict__ rho, float2 *__restrict__ u_out, int write_state, int do_scan, int apply_mask) {
    extern __shared__ float2 sm2[];
    const int r = blockIdx.x, Nt = a.Nt;
    float2 *b0 = sm2, *b1 = sm2 + Nt;
    load_mw_row(b0, r, a, F32, D, apply_mask ? __ldg(&a.mask_r[r]) : 1.0f);
    __syncthreads();
    if (write_state) store_state_row(b0, r, a, F32, Fb);
    if (!do_scan && !u_out) return;
    float2 *R = fft_row<true>(b0, b1, Nt, a.logNt, a.tw);
    const float inv = 1.0f / (float)Nt;
    if (u_out) {
        float2 *g = u_out + (size_t)r * Nt;
        for (int t = threadIdx.x; t < Nt; t += blockDim.x) g[t] = c_scale(R[t], inv);
    }
    if (!do_scan) return;
    float *sI = (float *)(R == b0 ? b1 : b0), *sW = sI + Nt;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        float2 v = c_scale(R[t], inv);
        sI[t] = fmaf(v.x, v.x, v.y * v.y) * a.sc.invE2;
    }
    __syncthreads();
    float *sx = (float *)R, *sJ = sx + Nt, *sB = (float *)(sm2 + 2 * Nt);
    scan_row(sI, sW, sx, sJ, sB, Nt, a.sc, a.lut, 0.0f, a.stats);
    float *gr = rho + (size_t)r * Nt;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) gr[t] = sx[t];
}

static cudaError_t set_smem(const void *fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t launch_row_entry(const RowFusedArgs &a, const float2 *u, float *F32, __nv_bfloat16 *Fb, float *rho,
                             int do_scan, cudaStream_t st) {
    size_t smem = 20 * (size_t)a.Nt;  // 2 complex buffers + one float scan array
    cudaError_t e = set_smem((const void *)k_row_entry, smem);
    if (e != cudaSuccess) return e;
    k_row_entry<<<a.Nr, NLSE_ROW_THREADS, smem, st>>>(a, u, F32, Fb, rho, do_scan);
    return cudaGetLastError();
}

cudaError_t launch_row_nl(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, const float *rho,
                          cudaStream_t st) {
    size_t smem = 16 * (size_t)a.Nt;
    cudaError_t e = set_smem((const void *)k_row_nl, smem);
    if (e != cudaSuccess) return e;
    k_row_nl<<<a.Nr, NLSE_ROW_THREADS, smem, st>>>(a, F32, Fb, D, rho);
    return cudaGetLastError();
}

cudaError_t launch_row_next(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, float *rho,
                            float2 *u_out, int write_state, int do_scan, int apply_mask, cudaStream_t st) {
    size_t smem = 20 * (size_t)a.Nt;
    cudaError_t e = set_smem((const void *)k_row_next, smem);
    if (e != cudaSuccess) return e;
    k_row_next<<<a.Nr, NLSE_ROW_THREADS, smem, st>>>(a, F32, Fb, D, rho, u_out, write_state, do_scan, apply_mask);
    return cudaGetLastError();
}

// FP32 planar field -> BF16 hi/lo terms (diagnostic path of nlse_debug_operator_product).
__global__ void k_split_field(const float *__restrict__ w, __nv_bfloat16 *__restrict__ Fb, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = w[i];
        __nv_bfloat16 h = __float2bfloat16_rn(v);
        Fb[i] = h;
        Fb[n + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

cudaError_t launch_split_field(const float *w, __nv_bfloat16 *Fb, size_t n, cudaStream_t st) {
    k_split_field<<<1024, 256, 0, st>>>(w, Fb, n);
    return cudaGetLastError();
}
