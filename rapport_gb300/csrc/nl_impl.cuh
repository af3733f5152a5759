// Pointwise nonlinear-step math shared by the elementwise and the fused row kernels.
// (See k_nonlinear.cu for the derivation from NonlinearOperator.split.)
#pragma once
#include "nlse_internal.cuh"


static __constant__ float c_pow10[18] = {1e0f,  1e1f,  1e2f,  1e3f,  1e4f,  1e5f,  1e6f,  1e7f,  1e8f,
                                  1e9f,  1e10f, 1e11f, 1e12f, 1e13f, 1e14f, 1e15f, 1e16f, 1e17f};

static __constant__ float c_ipow10[18] = {1e0f,   1e-1f,  1e-2f,  1e-3f,  1e-4f,  1e-5f,  1e-6f,  1e-7f,  1e-8f,
                                          1e-9f,  1e-10f, 1e-11f, 1e-12f, 1e-13f, 1e-14f, 1e-15f, 1e-16f, 1e-17f};

// photo-ionisation loss rate [1/m] before depletion, for a finite I >= 0.
// Interval of the knots 10^d (1 + 0.01 m) holding clip(I): the decade from a
// fast log10 corrected against the exact powers, m by one multiply; the
// position s in the interval; the per-interval Hermite cubic (pre-scaled by
// Kc invE2 / x_i); times x_i / (I + 1e-30 invE2).
__device__ __forceinline__ float photo_rate(float I, const NLParams &p, const float4 *__restrict__ tab) {
    const float Ic = fminf(fmaxf(I, p.Imin), p.Imax);
    int d = min(max(__float2int_rd(__log10f(Ic)), 0), 16);
    if (Ic < c_pow10[d]) d = max(d - 1, 0);
    else if (Ic >= c_pow10[d + 1]) d = min(d + 1, 16);
    const float p10 = c_pow10[d], ip10 = c_ipow10[d];
    int m = __float2int_rz(fmaf(Ic, ip10, -1.0f) * 100.0f);
    m = min(max(m, 0), min(899, p.n_int - 1 - 900 * d));
    const float xi = p10 * fmaf(0.01f, (float)m, 1.0f);
    const float s = (Ic - xi) * (100.0f * ip10);
    const float4 cf = __ldg(&tab[900 * d + m]);
    const float V = fabsf(fmaf(s, fmaf(s, fmaf(s, cf.w, cf.z), cf.y), cf.x));
    return V * __fdividef(xi, I + p.tiny_I);
}

// u e^{x} for x <= 0 (the alpha/2 damping) as u + u (e^{x} - 1): the factor's
// error is then relative to e^{x} - 1, not to 1, so a weakly absorbed point
// is not biased by the same expf rounding every z-step.
__device__ __forceinline__ float2 c_damp(float2 u, float x) {
    if (x == 0.0f) return u;  // no absorption (no carriers, negligible photo-ionisation)
    const float m = expm1f(x);
    return make_float2(fmaf(u.x, m, u.x), fmaf(u.y, m, u.y));
}

// alpha(u, rho) and the raw sum it clamps, as split() computes them.
__device__ __forceinline__ float alpha_of(float a2, float rho, const NLParams &p,
                                          const float4 *__restrict__ tab, float *raw) {
    float photo = 0.0f;
    if (p.photo_on) {
        const float I = a2 * p.invE2;
        // one test on the common path (a finite I below I_skip); NaN fails it too
        if (!(I < p.I_skip)) {
            if (isfinite(I)) {
                float dep = fminf(fmaxf((p.rho_max - rho) * p.inv_rho_max, 0.0f), 1.0f);
                photo = photo_rate(I, p, tab) * dep;
            } else if (isnan(I)) {
                photo = I;  // NaN: split() turns the sum into alpha = 0 (nan_to_num)
            }             // +Inf: W(Imax) / Inf = 0 in split()
        }
    }
    float ar = fmaf(p.pp_abs, rho, photo);
    *raw = ar;
    return isfinite(ar) ? fmaxf(ar, 0.0f) : 0.0f;
}

// RK right-hand side of split() for one point; rho, rho_s frozen.
__device__ __forceinline__ float2 nl_rhs(float2 u, float rho, float rho_s, const NLParams &p,
                                         const float4 *__restrict__ tab) {
    float a2 = fmaf(u.x, u.x, u.y * u.y);
    float w = fmaf(p.kp, a2, fmaf(p.ste_pref, rho_s, -p.pp_def * rho));  // i w u
    float corr = 0.0f;
    if (rho < 0.0f) {
        float raw;
        float al = alpha_of(a2, rho, p, tab, &raw);
        corr = isfinite(raw) ? al - raw : 0.0f;
    }
    float2 r = make_float2(fmaf(corr, u.x, -w * u.y), fmaf(corr, u.y, w * u.x));
    // zero below |u|^2 = 1e-30 (also NaN) and for a non-finite result, as a
    // select rather than an early return
    const bool keep = a2 >= 1e-30f && isfinite(r.x) && isfinite(r.y);
    return keep ? r : make_float2(0.0f, 0.0f);
}

__device__ __forceinline__ float2 nl_point(float2 u, float rho, float rho_s, float dz, const NLParams &p,
                                           const float4 *__restrict__ tab) {
    const float hdz = 0.5f * dz;
    float raw;
    float a = alpha_of(fmaf(u.x, u.x, u.y * u.y), rho, p, tab, &raw);
    u = c_damp(u, -hdz * a);
    float2 k1 = nl_rhs(u, rho, rho_s, p, tab);
    float2 k2 = nl_rhs(make_float2(fmaf(hdz, k1.x, u.x), fmaf(hdz, k1.y, u.y)), rho, rho_s, p, tab);
    float2 k3 = nl_rhs(make_float2(fmaf(hdz, k2.x, u.x), fmaf(hdz, k2.y, u.y)), rho, rho_s, p, tab);
    float2 k4 = nl_rhs(make_float2(fmaf(dz, k3.x, u.x), fmaf(dz, k3.y, u.y)), rho, rho_s, p, tab);
    const float s6 = dz * (1.0f / 6.0f);
    u.x = fmaf(s6, fmaf(2.0f, k2.x + k3.x, k1.x) + k4.x, u.x);
    u.y = fmaf(s6, fmaf(2.0f, k2.y + k3.y, k1.y) + k4.y, u.y);
    a = alpha_of(fmaf(u.x, u.x, u.y * u.y), rho, p, tab, &raw);
    return c_damp(u, -hdz * a);
}

