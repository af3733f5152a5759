// Full-physics split() kernels (Raman, self-steepening, space-time focusing):
// the alpha/2 + RK4 + alpha/2 block and split() itself, one CTA per row with
// the row's transforms in shared memory (fullnl_impl.cuh).  N_t <= 4096: the
// six complex rows of 4096 points take 198 KB of shared memory.
#include "fullnl_impl.cuh"

template <int NT>
__global__ void __launch_bounds__(full_threads<NT>(), full_min_blocks<NT>())
k_nl_full(float2 *__restrict__ u, const float *__restrict__ rho, const float *__restrict__ rhos, float dz, NLParams p,
          const float4 *__restrict__ tab, FullTabs ft, const float2 *__restrict__ tw) {
    extern __shared__ float2 smf[];
    // the constants the out-of-line right-hand side reads at every point: a shared copy
    __shared__ NLParams s_nl;
    __shared__ FullTabs s_ft;
    if (threadIdx.x == 0) {
        s_nl = p;
        s_ft = ft;
    }
    const FullRows m = full_rows<NT>(smf);
    const size_t base = (size_t)blockIdx.x * NT;
    for (int t = threadIdx.x; t < NT; t += full_threads<NT>()) m.U[t] = u[base + t];
    __syncthreads();
    nl_block_full<NT>(m, rho + base, rhos ? rhos + base : nullptr, dz, s_nl, tab, s_ft, tw);
    for (int t = threadIdx.x; t < NT; t += full_threads<NT>()) u[base + t] = m.U[t];
}

template <int NT>
__global__ void __launch_bounds__(full_threads<NT>(), full_min_blocks<NT>())
k_split_full(const float2 *__restrict__ u, const float *__restrict__ rho, const float *__restrict__ rhos,
             float2 *__restrict__ rhs, float *__restrict__ alpha, NLParams p, const float4 *__restrict__ tab,
             FullTabs ft, const float2 *__restrict__ tw) {
    extern __shared__ float2 smf[];
    // the constants the out-of-line right-hand side reads at every point: a shared copy
    __shared__ NLParams s_nl;
    __shared__ FullTabs s_ft;
    if (threadIdx.x == 0) {
        s_nl = p;
        s_ft = ft;
    }
    const FullRows m = full_rows<NT>(smf);
    const size_t base = (size_t)blockIdx.x * NT;
    for (int t = threadIdx.x; t < NT; t += full_threads<NT>()) {
        const float2 v = u[base + t];
        m.S[t] = v;
        if (alpha) {
            const float r = rho[base + t];
            alpha[base + t] = alpha_from(photo_term(fmaf(v.x, v.x, v.y * v.y), r, p, tab), r, p);
        }
    }
    __syncthreads();
    const float2 *K = rhs_full<NT>(m, rho + base, rhos ? rhos + base : nullptr, s_nl, tab, s_ft, tw);
    for (int t = threadIdx.x; t < NT; t += full_threads<NT>()) rhs[base + t] = K[pidx(t)];
}

static FullTabs ctx_tabs(const nlse_ctx *c) {
    return FullTabs{c->d_Tss, c->d_invUnl, c->d_Rf, c->raman_z, c->raman_amp, c->raman_iir};
}

cudaError_t launch_nl_full(nlse_ctx *c, float2 *u, const float *rho, const float *rho_s, float dz,
                           cudaStream_t st) {
    NLSE_DISPATCH_NT_FULL(c->logNt, {
        const size_t smem = full_smem_bytes<NT>();
        cudaError_t e = cudaFuncSetAttribute(k_nl_full<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_nl_full<NT><<<c->Nr, full_threads<NT>(), smem, st>>>(u, rho, rho_s, dz, c->nl, c->d_pchip, ctx_tabs(c),
                                                            c->d_tw);
    });
    return cudaGetLastError();
}

cudaError_t launch_split_full(nlse_ctx *c, const float2 *u, const float *rho, const float *rho_s, float2 *rhs,
                              float *alpha, cudaStream_t st) {
    NLSE_DISPATCH_NT_FULL(c->logNt, {
        const size_t smem = full_smem_bytes<NT>();
        cudaError_t e =
            cudaFuncSetAttribute(k_split_full<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_split_full<NT><<<c->Nr, full_threads<NT>(), smem, st>>>(u, rho, rho_s, rhs, alpha, c->nl, c->d_pchip,
                                                               ctx_tabs(c), c->d_tw);
    });
    return cudaGetLastError();
}
