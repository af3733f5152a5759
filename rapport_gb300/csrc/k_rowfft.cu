// Row FFT kernels: the spectral part of the linear half step.
//
// LinearOperator.half_linear (operators.py:47-53) applies, between the two
// Hankel products, fft_t -> multiply by exp(i phase) * spec_mask -> ifft_t with
// phase = (delta_k(Omega) - rho_m^2 / (2 k0)) dz / 2 (space-time focusing off,
// so the phase separates into an Omega factor and a Hankel-mode factor).
// Here one CTA owns one row (one Hankel mode m): it loads the row into shared
// memory, runs the forward FFT, multiplies by Pr[m] * Pt[Omega], runs the
// inverse FFT and stores the row -- one HBM read and one write per element.
#include "nlse_internal.cuh"

// Per-dz phase tables, computed in FP64 on the device and rounded once:
//   Pt[k]  = exp(i delta_k[k] dz/2) * spec_mask[k] * Rk*iRk / Nt   (1/Nt = ifft norm)
//   Ptf[k] = the same without 1/Nt (split path; may be NULL), and in
//            Ptf[Nt + k] its FP32 rounding remainder (P - (float)P)
//   Pr[m]  = exp(-i rho_m^2 dz / (4 k0))
__global__ void k_phase_tables(const double *__restrict__ delta_k, const double *__restrict__ spec_mask,
                               const double *__restrict__ rho_modes, int Nt, int Nr, double dz,
                               double komega, double scale, float2 *__restrict__ Pt,
                               float2 *__restrict__ Pr, float2 *__restrict__ Ptf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Nt) {
        double s, c;
        sincos(delta_k[i] * dz * 0.5, &s, &c);
        double m = spec_mask[i] * scale / (double)Nt;
        Pt[i] = make_float2((float)(c * m), (float)(s * m));
        if (Ptf) {
            // split-BF16 path: FP32 value and its rounding remainder (Ptf[Nt + i])
            const double mf = spec_mask[i] * scale, pr = c * mf, pi = s * mf;
            const float2 h = make_float2((float)pr, (float)pi);
            Ptf[i] = h;
            Ptf[Nt + i] = make_float2((float)(pr - (double)h.x), (float)(pi - (double)h.y));
        }
    }
    if (i < Nr) {
        double s, c;
        double r = rho_modes[i];
        sincos(-r * r * dz / (4.0 * komega), &s, &c);
        Pr[i] = make_float2((float)c, (float)s);
    }
}

cudaError_t launch_phase_tables(nlse_ctx *c, double dz, cudaStream_t stream) {
    int n = c->Nt > c->Nr ? c->Nt : c->Nr;
    k_phase_tables<<<(n + 255) / 256, 256, 0, stream>>>(c->d_delta_k, c->d_spec_mask, c->d_rho_modes,
                                                        c->Nt, c->Nr, dz, c->komega, c->Rk_iRk,
                                                        c->d_Pt, c->d_Pr, c->d_Ptf);
    return cudaGetLastError();
}

// With space-time focusing the diffraction phase depends on Omega through
// U^-1 (operators.py:50), so it no longer separates: per dz the whole table
//   P2[m, k] = exp(i (delta_k[k] - rho_m^2 invU[k] / (2 k0)) dz/2) spec_mask[k] Rk iRk / Nt
// is built in FP64 and rounded once (8 Nr Nt bytes, allocated only then).
__global__ void k_phase_table_2d(const double *__restrict__ delta_k, const double *__restrict__ spec_mask,
                                 const double *__restrict__ rho_modes, const double *__restrict__ inv_U, int Nt,
                                 int Nr, double dz, double komega, double scale, float2 *__restrict__ P2) {
    const size_t n = (size_t)Nr * Nt;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int m = (int)(i / Nt), k = (int)(i % Nt);
        const double r = rho_modes[m];
        double s, c;
        sincos((delta_k[k] - r * r / (2.0 * komega) * inv_U[k]) * dz * 0.5, &s, &c);
        const double a = spec_mask[k] * scale / (double)Nt;
        P2[i] = make_float2((float)(c * a), (float)(s * a));
    }
}

cudaError_t launch_phase_table_2d(nlse_ctx *c, double dz, cudaStream_t stream) {
    k_phase_table_2d<<<4 * 152, 256, 0, stream>>>(c->d_delta_k, c->d_spec_mask, c->d_rho_modes, c->d_invUop, c->Nt,
                                                   c->Nr, dz, c->komega, c->Rk_iRk, c->d_P2);
    return cudaGetLastError();
}

// u[m, :] <- ifft( Pr[m] Pt * fft(u[m, :]) ), one CTA per row, in place
// (P2 given: ifft( P2[m, :] * fft(u[m, :]) )).
template <int NT>
__global__ void __launch_bounds__(NLSE_ROW_THREADS)
k_fft_phase_ifft(float2 *__restrict__ u, const float2 *__restrict__ tw, const float2 *__restrict__ Pt,
                 const float2 *__restrict__ Pr, const float2 *__restrict__ P2) {
    extern __shared__ float2 smem[];
    float2 *b0 = smem, *b1 = smem + fft_slots(NT);
    const size_t row = blockIdx.x;
    float2 *g = u + row * (size_t)NT;
    for (int i = threadIdx.x; i < NT; i += blockDim.x) b0[pidx(i)] = g[i];
    __syncthreads();
    float2 *s = fft_row<NT, false>(b0, b1, tw);
    if (P2) {
        const float2 *q = P2 + row * (size_t)NT;
        for (int i = threadIdx.x; i < NT; i += blockDim.x) s[pidx(i)] = c_mul(s[pidx(i)], __ldg(&q[i]));
    } else {
        const float2 pr = Pr[row];
        for (int i = threadIdx.x; i < NT; i += blockDim.x) s[pidx(i)] = c_mul(s[pidx(i)], c_mul(pr, __ldg(&Pt[i])));
    }
    __syncthreads();
    float2 *r = fft_row<NT, true>(s, s == b0 ? b1 : b0, tw);
    for (int i = threadIdx.x; i < NT; i += blockDim.x) g[i] = r[pidx(i)];
}

static cudaError_t fft_phase_ifft(float2 *u, int Nr, int logNt, const float2 *tw, const float2 *Pt,
                                  const float2 *Pr, const float2 *P2, cudaStream_t stream) {
    NLSE_DISPATCH_NT(logNt, {
        const size_t smem = 2 * (size_t)fft_slots(NT) * sizeof(float2);
        cudaError_t e = cudaFuncSetAttribute(k_fft_phase_ifft<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        k_fft_phase_ifft<NT><<<Nr, NLSE_ROW_THREADS, smem, stream>>>(u, tw, Pt, Pr, P2);
    });
    return cudaGetLastError();
}

cudaError_t launch_fft_phase_ifft(nlse_ctx *c, float2 *u, cudaStream_t stream) {
    return fft_phase_ifft(u, c->Nr, c->logNt, c->d_tw, c->d_Pt, c->d_Pr, c->d_P2, stream);
}

// The same row kernel on caller-provided tables (used by the allocation-free entry point).
cudaError_t launch_fft_phase_ifft_tables(float2 *u, int Nr, int Nt, int logNt, const float2 *tw, const float2 *Pt,
                                         const float2 *Pr, cudaStream_t stream) {
    (void)Nt;
    return fft_phase_ifft(u, Nr, logNt, tw, Pt, Pr, nullptr, stream);
}
