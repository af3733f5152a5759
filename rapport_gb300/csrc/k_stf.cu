// Space-time focusing in the tensor-core forms.
//
// With space-time focusing the reference's half step (operators.py:47-53)
//     iRk Y ifft_t( e^{i (dk(W) - rho_m^2 U^-1(W) / (2 k0)) dz/2} mask fft_t( Rk Y u ) )
// has a radial phase that depends on the frequency W (grids.py:88-111), so
// Y diag(P_r) Y is a different matrix for every column and does not merge
// into one operator.  In the Omega domain the split forms therefore run the
// reference's own factorisation, on the tensor cores, for the correction
// E(W) = Y diag(P2 - 1) Y of M(W) = I + E(W) (Y Y = I):
//     G1  v  = Y w                       (both planes; block-diagonal product)
//     ph  v' = (P2(rho_m, W_t) - 1) v    (this file: one pass, FP16 terms out)
//     G2  D  = Y v'
//     row x  = P_t (w + D)               (the row kernels; w exact in FP32)
// with P2 = e^{-i rho_m^2 dz U^-1(W_t) / (4 k0)}.  As in the merged form only
// the correction passes through FP16: carrying the whole field through four
// FP16 roundings per z-step left its values far below the peak near FP16's
// exponent floor (~17 bits), rounded the same way step after step -- a
// systematic drift of ~1e-5 per step.  Y is split into 3 scaled FP16 terms
// (~33 bits), of which the products read the first two (~22 bits: as accurate
// over 0.5 cm as three, since only the correction passes through them), the
// field and v' in 2 (~22 bits).  P2 - 1 is built in FP64 per dz (cos - 1 as -2 sin^2 of the
// half angle) and applied with its FP32 rounding remainder folded in.  The
// FP16 scale of v' follows its measured maxima.
#include "nlse_internal.cuh"

// diag(Y, Y) 2^sa as 3 FP16 terms (h + m + l), stacked term-major like E'.
__global__ void k_split_Yb16(const double *__restrict__ Y, int Nr, int Nrp, int sa, __half *__restrict__ A,
                             int *__restrict__ scale) {
    const size_t K2 = 2 * (size_t)Nrp, total = K2 * K2;
    const double sc = ldexp(1.0, sa);
    if (blockIdx.x == 0 && threadIdx.x == 0) scale[NLSE_SC_SA] = sa;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t m = i / K2, k = i % K2;
        const size_t mr = m % Nrp, kr = k % Nrp;
        const bool same = (m >= (size_t)Nrp) == (k >= (size_t)Nrp);
        const double v = (same && mr < (size_t)Nr && kr < (size_t)Nr) ? Y[mr * Nr + kr] * sc : 0.0;
        const __half h = __double2half(v);
        const double r1 = v - (double)__half2float(h);
        const __half mm = __double2half(r1);
        const __half l = __double2half(r1 - (double)__half2float(mm));
        A[i] = h;
        A[total + i] = mm;
        A[2 * total + i] = l;
    }
}

cudaError_t launch_split_Yb16(const double *Y64, int Nr, int Nrp, int sa, __half *A, int *scale,
                              cudaStream_t stream) {
    k_split_Yb16<<<1024, 256, 0, stream>>>(Y64, Nr, Nrp, sa, A, scale);
    return cudaGetLastError();
}

__global__ void k_stf_table(const double *__restrict__ rho, const double *__restrict__ invU, int Nr, int Nt,
                            double dz, double komega, float4 *__restrict__ P2s) {
    const size_t n = (size_t)Nr * Nt;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int m = (int)(i / Nt), t = (int)(i % Nt);
        const double r = rho[m];
        const double ph = -r * r * dz * invU[t] / (4.0 * komega);
        const double h = sin(0.5 * ph), c = -2.0 * h * h, s = sin(ph);  // e^{i ph} - 1
        const float hc = (float)c, hs = (float)s;
        P2s[i] = make_float4(hc, hs, (float)(c - (double)hc), (float)(s - (double)hs));
    }
}

cudaError_t launch_stf_table(const double *rho, const double *invU, int Nr, int Nt, double dz, double komega,
                             float4 *P2s, cudaStream_t stream) {
    k_stf_table<<<4 * 152, 256, 0, stream>>>(rho, invU, Nr, Nt, dz, komega, P2s);
    return cudaGetLastError();
}

// v' = P2s v for one point (v = D 2^-(sa + sb) as complex)
__device__ __forceinline__ float2 stf_point(float dr, float di, float ds, float4 p) {
    return c_mul_comp(make_float2(dr * ds, di * ds), make_float2(p.x, p.y), make_float2(p.z, p.w));
}

// Input g (g % 6 == 0): the largest component of this input's own v', into the
// ring slot it takes its scale from (the phase pass then uses it directly).
__global__ void k_stf_absmax(const float *__restrict__ D, const float4 *__restrict__ P2s, int Nr, int Nrp, int Nt,
                             int g, int *__restrict__ scale) {
    const int sa = __ldcg(&scale[NLSE_SC_SA]), sb = __ldcg(&scale[NLSE_SC_SB + g % 2]);
    const float ds = ldexpf(1.0f, -(sa + sb));
    const size_t plane = (size_t)Nr * Nt;
    float mx = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
        // point i = m Nt + t of rows m < Nr: Re plane at i, Im plane Nrp rows further
        const float2 v = stf_point(D[i], D[(size_t)Nrp * Nt + i], ds, __ldg(P2s + i));
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&scale[NLSE_SC_VMAX + (g + 2) % 3], __float_as_int(mx));
}

// One CTA per radius m < Nr: v = (D[m], D[Nrp + m]) 2^-(sa + sb_g), v' = P2s v,
// stored as the FP16 hi / lo terms of v' 2^sv in the planes of Fb.  The scale
// maps the previous input's largest |component of v'| below 2^7 (512x
// headroom before FP16's 65504; an overflow is counted), and this input's
// largest component goes to its ring slot for the next.
__global__ void __launch_bounds__(256) k_stf_phase(const float *__restrict__ D, const float4 *__restrict__ P2s,
                                                   __half *__restrict__ Fb, int Nrp, int Nt, int g,
                                                   int *__restrict__ scale) {
    const int m = blockIdx.x;
    const int sa = __ldcg(&scale[NLSE_SC_SA]), sb = __ldcg(&scale[NLSE_SC_SB + g % 2]);
    const float ds = ldexpf(1.0f, -(sa + sb));
    const float prev = __int_as_float(__ldcg(&scale[NLSE_SC_VMAX + (g + 2) % 3]));
    int e = 0;
    if (prev > 0.0f && isfinite(prev)) frexpf(prev, &e);
    const int sv = min(max(7 - e, -100), 100);
    const float sc = ldexpf(1.0f, sv);
    const size_t rows = 2 * (size_t)Nrp;
    const float *dr = D + (size_t)m * Nt, *di = D + ((size_t)Nrp + m) * Nt;
    const float4 *p = P2s + (size_t)m * Nt;
    __half *hre = Fb + (size_t)m * Nt, *him = Fb + ((size_t)Nrp + m) * Nt;
    __half *lre = hre + rows * Nt, *lim = him + rows * Nt;
    float mx = 0.0f;
    for (int t = 2 * threadIdx.x; t < Nt; t += 2 * blockDim.x) {
        const float2 xr = *reinterpret_cast<const float2 *>(dr + t), xi = *reinterpret_cast<const float2 *>(di + t);
        const float4 p0 = __ldg(p + t), p1 = __ldg(p + t + 1);
        const float2 v0 = stf_point(xr.x, xi.x, ds, p0), v1 = stf_point(xr.y, xi.y, ds, p1);
        mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v0.x), fabsf(v0.y)), fmaxf(fabsf(v1.x), fabsf(v1.y))));
        const float x0 = v0.x * sc, x1 = v1.x * sc, y0 = v0.y * sc, y1 = v1.y * sc;
        const __half2 hx = __floats2half2_rn(x0, x1), hy = __floats2half2_rn(y0, y1);
        *reinterpret_cast<__half2 *>(hre + t) = hx;
        *reinterpret_cast<__half2 *>(him + t) = hy;
        *reinterpret_cast<__half2 *>(lre + t) = __floats2half2_rn(x0 - __low2float(hx), x1 - __high2float(hx));
        *reinterpret_cast<__half2 *>(lim + t) = __floats2half2_rn(y0 - __low2float(hy), y1 - __high2float(hy));
    }
    // a finite value above 65504 after scaling overflowed its FP16 term
    const int ovf = __syncthreads_or(isfinite(mx) && !(mx * sc <= 65504.0f));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&scale[NLSE_SC_VMAX + g % 3], __float_as_int(mx));
    if (threadIdx.x == 0) {
        if (ovf) atomicAdd(&scale[NLSE_SC_OVF], 1);
        if (m == 0) {
            scale[NLSE_SC_VB + g % 2] = sv;
            scale[NLSE_SC_VMAX + (g + 1) % 3] = 0;  // the slot input g + 1 will fill
        }
    }
}

cudaError_t launch_stf_phase(const float *D, const float4 *P2s, __nv_bfloat16 *Fb, int Nr, int Nrp, int Nt, float cY,
                             int g, int *scale, cudaStream_t stream) {
    (void)cY;
    // every sixth input (the period of all the scale rings, and of a batch's
    // captured z-steps) takes its scale from its own v' instead of the previous
    // input's, so every call starts from a measured scale
    if (g % 6 == 0) {
        cudaError_t e = cudaMemsetAsync(scale + NLSE_SC_VMAX, 0, 3 * sizeof(int), stream);
        if (e != cudaSuccess) return e;
        k_stf_absmax<<<2 * 152, 256, 0, stream>>>(D, P2s, Nr, Nrp, Nt, g, scale);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_stf_phase<<<Nr, 256, 0, stream>>>(D, P2s, reinterpret_cast<__half *>(Fb), Nrp, Nt, g, scale);
    return cudaGetLastError();
}
