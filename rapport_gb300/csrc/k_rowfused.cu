// Runtime dispatch of the fused row kernels over N_t (the kernels and their
// per-N_t launchers are in k_rowfused.cuh, instantiated in k_row_n*.cu), and
// the small helper kernels of the split forms.
#include "k_rowfused.cuh"

cudaError_t launch_row_entry(const RowFusedArgs &a, const float2 *u, float *F32, __nv_bfloat16 *Fb, float *rho,
                             int do_scan, cudaStream_t st) {
    NLSE_DISPATCH_NT(a.logNt, return RowKernels<NT>::entry(a, u, F32, Fb, rho, do_scan, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_nl_full(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                               const float *rho, int g, cudaStream_t st) {
    NLSE_DISPATCH_NT_FULL(a.logNt, return RowKernels<NT>::nl_full(a, F32, Fb, D, rho, g, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_nl(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, const float *rho,
                          int g, cudaStream_t st) {
    NLSE_DISPATCH_NT(a.logNt, return RowKernels<NT>::nl(a, F32, Fb, D, rho, g, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_next(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, float *rho,
                            float2 *u_out, int write_state, int do_scan, int apply_mask, int g, cudaStream_t st) {
    NLSE_DISPATCH_NT(a.logNt,
                     return RowKernels<NT>::next(a, F32, Fb, D, rho, u_out, write_state, do_scan, apply_mask, g, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_batch(int kind, int logNt, const BatchPulse *P, const int2 *work, int nblocks, int flag,
                             int g, cudaStream_t st) {
    if (kind == 3) {
        NLSE_DISPATCH_NT_FULL(logNt, return RowKernels<NT>::batch(kind, P, work, nblocks, flag, g, st));
    } else {
        NLSE_DISPATCH_NT(logNt, return RowKernels<NT>::batch(kind, P, work, nblocks, flag, g, st));
    }
    return cudaErrorInvalidValue;
}

// Split-FP16 form: before the entry kernel writes GEMM input 0 = F[u], its
// "previous maximum" is the bound Nt max |u| >= max |F[u]| (slot 2), and the
// slot input 0 fills is cleared.
__global__ void k_field_bound(const float2 *__restrict__ u, size_t n, int Nt, int *__restrict__ scale) {
    float mx = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = u[i];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    mx = block_max(mx);
    if (threadIdx.x == 0) atomicMax(&scale[NLSE_SC_MAX + 2], __float_as_int(mx * (float)Nt * 1.5f));
}

cudaError_t launch_field_bound(const float2 *u, size_t n, int Nt, int *scale, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(scale + NLSE_SC_MAX, 0, 3 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    k_field_bound<<<2 * 152, NLSE_ROW_THREADS, 0, st>>>(u, n, Nt, scale);
    return cudaGetLastError();
}

// FP32 planar field -> BF16 hi/lo terms (diagnostic path of nlse_debug_operator_product).
__global__ void k_split_field(const float *__restrict__ w, __nv_bfloat16 *__restrict__ hi, size_t lo_off,
                              size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = w[i];
        __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        hi[lo_off + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

cudaError_t launch_split_field(const float *w, __nv_bfloat16 *hi, size_t lo_off, size_t n, cudaStream_t st) {
    k_split_field<<<1024, 256, 0, st>>>(w, hi, lo_off, n);
    return cudaGetLastError();
}
