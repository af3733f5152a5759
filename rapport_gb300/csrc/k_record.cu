// Per-plane diagnostics of Integrator._record (integrator.py:179-224), on the device.
//
// The reference computes them with ~20 CuPy reductions and a loss_rates()
// PCHIP pass per saved plane.  Here one CTA per radius reduces its row once,
// accumulating in FP64:
//   out[r][0] = sum_t |u|^2                       (fluence / (dt invE2))
//   out[r][1] = max_t rho        out[r][2] = max_t rho_s
//   out[r][3] = max_t |u|^2                       (peak intensity / invE2)
//   out[r][4] = sum_t 2 photo |u|^2               (photo-ionisation loss)
//   out[r][5] = sum_t 2 plasma |u|^2              (plasma absorption loss)
//   out[r][6 + b] = sum_{t in bin b} 2 (photo + plasma) |u|^2
// photo and plasma are the loss rates of NonlinearOperator.loss_rates
// (operators.py:148-163); the host applies dt, invE2 and the unit factors.
#include "nl_impl.cuh"

#define REC_FIXED 6

__global__ void __launch_bounds__(256)
k_record(const float2 *__restrict__ u, const float *__restrict__ rho, const float *__restrict__ rho_s, int Nt,
         NLParams p, const float4 *__restrict__ tab, const int *__restrict__ bin_of_t, int nbins,
         double *__restrict__ out) {
    const int r = blockIdx.x;
    const size_t base = (size_t)r * Nt;
    const int nf = REC_FIXED + nbins;
    double acc[REC_FIXED + 8];
    for (int f = 0; f < nf; ++f) acc[f] = 0.0;
    float rmax = 0.0f, smax = 0.0f, imax = 0.0f;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        const float2 v = u[base + t];
        const float a2 = fmaf(v.x, v.x, v.y * v.y);
        const float rh = rho[base + t];
        rmax = fmaxf(rmax, rh);
        if (rho_s) smax = fmaxf(smax, rho_s[base + t]);
        imax = fmaxf(imax, a2);
        float photo = 0.0f;
        const float I = a2 * p.invE2;
        if (p.photo_on && isfinite(I)) {
            const float dep = fminf(fmaxf((p.rho_max - rh) * p.inv_rho_max, 0.0f), 1.0f);
            photo = photo_rate(I, p, tab) * dep;
        }
        const float plasma = p.pp_abs * rh;
        const double w = 2.0 * (double)a2;
        acc[0] += (double)a2;
        acc[4] = fma(w, (double)photo, acc[4]);
        acc[5] = fma(w, (double)plasma, acc[5]);
        if (nbins) {
            const int b = bin_of_t[t];
            if (b >= 0 && b < nbins) acc[REC_FIXED + b] = fma(w, (double)(photo + plasma), acc[REC_FIXED + b]);
        }
    }
    __shared__ double sred[8][REC_FIXED + 8];
    __shared__ float fred[8][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int f = 0; f < nf; ++f)
        for (int o = 16; o > 0; o >>= 1) acc[f] += __shfl_xor_sync(0xffffffffu, acc[f], o);
    for (int o = 16; o > 0; o >>= 1) {
        rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        smax = fmaxf(smax, __shfl_xor_sync(0xffffffffu, smax, o));
        imax = fmaxf(imax, __shfl_xor_sync(0xffffffffu, imax, o));
    }
    if (lane == 0) {
        for (int f = 0; f < nf; ++f) sred[wid][f] = acc[f];
        fred[wid][0] = rmax;
        fred[wid][1] = smax;
        fred[wid][2] = imax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        double tot[REC_FIXED + 8];
        float mx[3] = {0.0f, 0.0f, 0.0f};
        for (int f = 0; f < nf; ++f) tot[f] = 0.0;
        for (int w = 0; w < nw; ++w) {
            for (int f = 0; f < nf; ++f) tot[f] += sred[w][f];
            for (int k = 0; k < 3; ++k) mx[k] = fmaxf(mx[k], fred[w][k]);
        }
        double *o = out + (size_t)r * nf;
        o[0] = tot[0];
        o[1] = mx[0];
        o[2] = mx[1];
        o[3] = mx[2];
        o[4] = tot[4];
        o[5] = tot[5];
        for (int b = 0; b < nbins; ++b) o[REC_FIXED + b] = tot[REC_FIXED + b];
    }
}

cudaError_t launch_record(nlse_ctx *c, const float2 *u, const float *rho, const float *rho_s, const int *bin_of_t,
                          int nbins, double *out, cudaStream_t st) {
    if (nbins < 0 || nbins > 8) return cudaErrorInvalidValue;
    k_record<<<c->Nr, 256, 0, st>>>(u, rho, rho_s, c->Nt, c->nl, c->d_pchip, bin_of_t, nbins, out);
    return cudaGetLastError();
}
