// Carrier-rate march along t as a parallel scan (one CTA per radius).
//
// The reference kernel (kernels.py:36-106) gives each radius one thread that
// walks t = 0..Nt-2 sequentially: 4 CTAs at Nr = 1024, FP64, uncoalesced.  Per
// step n it maps
//     x_{n+1} = f_n(x_n) = e^{z} x_n + b_n d(x_n) phi1(z),   z = a_n d(x_n) - c
// with d(x) = clamp(1 - x/na, 0, 1), a_n = beta dt I_avg, b_n = dt W_avg,
// c = dt/tau_r, phi1(z) = (e^z - 1)/z, and clamps (non-finite/negative -> 0,
// x > na -> na).  f_n is nonlinear in x only through the depletion d(x).
//
// Here the recurrence is solved by Newton's method on the whole trajectory:
// linearising every f_n around the current iterate x^k gives an AFFINE
// recurrence x_{n+1} = J_n x_n + (f_n(x^k_n) - J_n x^k_n), which one
// block-wide scan of affine maps (thread-local sequential composition, warp
// shuffles, one smem exchange across warps) solves exactly.  Newton converges
// quadratically; the loop stops when the trajectory changes by less than
// 1e-6 of its maximum (2 sweeps when the depletion is negligible, <= 7 at
// 66 % depletion).  A non-finite average intensity makes f_n == 0 (the
// reference's NaN -> 0 reset), which the affine form represents exactly
// (J = 0, B = 0).  A row that hits the x > na clamp or does not converge is
// re-marched sequentially in FP32 by one thread -- bit-for-bit the reference
// recurrence, just slow -- so saturated rows stay correct.
//
// Per point: 8 B of field read, 4 B of density written (HBM); the iterations
// run out of shared memory.
#include "scan_impl.cuh"

// Threads a row: 256, 512 from N_t = 2048 and 1024 from 8192 -- at most 8
// steps a thread, so long rows keep short sequential chunks, and 16-32 warps
// per CTA where the scan arrays leave room for only one or two CTAs per SM.
static int scan_threads(int Nt) { return Nt >= 8192 ? 1024 : (Nt >= 2048 ? 512 : NLSE_ROW_THREADS); }

__global__ void __launch_bounds__(1024)
k_rate_scan(const float2 *__restrict__ u, float *__restrict__ rho, float *__restrict__ rho_s, int Nt,
            ScanParams p, const float *__restrict__ lut, const float *__restrict__ lut_s, int zero_first,
            int *__restrict__ stats) {
    extern __shared__ float sm[];
    if (p.ste) {
        // two populations: sI sW sWs se ss + J (4) + B (2) arrays
        const int S = scan_span(Nt, blockDim.x);
        const ScanLayout L = scan_layout(Nt);
        const size_t row = blockIdx.x;
        const float2 *g = u + row * (size_t)Nt;
        float *ge = rho + row * (size_t)Nt, *gs = rho_s + row * (size_t)Nt;
        float x0e = 0.0f, x0s = 0.0f;
        if (!zero_first) {
            x0e = ge[0];
            x0s = gs[0];
            if (!isfinite(x0e) || x0e < 0.0f) x0e = 0.0f;
            if (!isfinite(x0s) || x0s < 0.0f) x0s = 0.0f;
        }
        float *sI = sm;
        for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
            float2 v = g[t];
            sI[scan_slot(t, L)] = fmaf(v.x, v.x, v.y * v.y) * p.invE2;
        }
        __syncthreads();
        float *jm[4] = {sm + 5 * S, sm + 6 * S, sm + 7 * S, sm + 8 * S};
        float *jb[2] = {sm + 9 * S, sm + 10 * S};
        scan_row2(sI, sm + S, sm + 2 * S, sm + 3 * S, sm + 4 * S, jm, jb, Nt, p, lut, lut_s, x0e, x0s, stats);
        for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
            if (t == 0 && !zero_first) continue;
            const int q = scan_slot(t, L);
            ge[t] = t == 0 ? 0.0f : sm[3 * S + q];
            gs[t] = t == 0 ? 0.0f : sm[4 * S + q];
        }
        return;
    }
    const int S = scan_span(Nt, blockDim.x);
    const ScanLayout L = scan_layout(Nt);
    float *sI = sm;
    const size_t row = blockIdx.x;
    const float2 *g = u + row * (size_t)Nt;
    float *grho = rho + row * (size_t)Nt;
    float x0 = 0.0f;
    if (!zero_first) {
        x0 = grho[0];
        if (!isfinite(x0) || x0 < 0.0f) x0 = 0.0f;
    }
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        float2 v = g[t];
        sI[scan_slot(t, L)] = fmaf(v.x, v.x, v.y * v.y) * p.invE2;
    }
    __syncthreads();
    float *sx = sm + 2 * S;
    scan_row(sI, sm + S, sx, sm + 3 * S, sm + 4 * S, Nt, p, lut, x0, stats);
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        if (t > 0 || zero_first) grho[t] = t == 0 ? 0.0f : sx[scan_slot(t, L)];
        if (rho_s && (t > 0 || zero_first)) rho_s[row * (size_t)Nt + t] = 0.0f;
    }
}

cudaError_t launch_rate_scan(nlse_ctx *c, const float2 *u, float *rho, float *rho_s, int zero_first,
                             cudaStream_t stream) {
    const int threads = scan_threads(c->Nt);
    size_t smem = (c->sc.ste ? 11 : 5) * (size_t)scan_span(c->Nt, threads) * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_rate_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_rate_scan<<<c->Nr, threads, smem, stream>>>(u, rho, rho_s, c->Nt, c->sc, c->d_lut_dt, c->d_lut_s_dt,
                                                           zero_first, c->d_flag);
    return cudaGetLastError();
}
