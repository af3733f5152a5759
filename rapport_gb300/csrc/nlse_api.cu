// C ABI of libnlse: context creation, table preparation and the drop-in
// entry points (declared and cross-referenced to the reference in include/nlse.h).
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "nlse_internal.cuh"

// FP16 terms of diag(Y, Y) the space-time-focusing products read (k_stf.cu
// writes three): two carry Y to ~22 bits, and the 0.5 cm error with space-time
// focusing is the same with two as with three (1.50e-5 against 1.52e-5
// relative L2), at 3 MMAs a k-slice instead of 4.
constexpr int NLSE_STF_Y_TERMS = 2;

static thread_local nlse_error_slot g_create_err;

// cuTensorMapEncodeTiled, resolved through the runtime so that the library
// itself does not link libcuda (it must load on hosts without a driver).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// Error of a context-free entry point, readable with nlse_get_last_error(NULL, ...).
void nlse_set_thread_error(int status, const char *msg) { nlse_set_error(&g_create_err, status, "%s", msg); }

void nlse_set_error(nlse_error_slot *slot, int status, const char *fmt, ...) {
    if (!slot) return;
    slot->status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(slot->msg, sizeof(slot->msg), fmt, ap);
    va_end(ap);
}

static void prof_free(nlse_ctx *c) {
    if (c->prof_ev) {
        for (int i = 0; i < 2 * c->prof_cap; ++i)
            if (c->prof_ev[i]) cudaEventDestroy(c->prof_ev[i]);
        free(c->prof_ev);
    }
    free(c->prof_kid);
    c->prof_ev = nullptr;
    c->prof_kid = nullptr;
    c->prof_on = c->prof_cap = c->prof_n = 0;
}

static void free_ctx(nlse_ctx *c) {
    if (!c) return;
    prof_free(c);
    void *ptrs[] = {c->d_tw,    c->d_Y,   c->d_Y64, c->d_rho_modes, c->d_delta_k, c->d_spec_mask,
                    c->d_mask_r, c->d_pchip, c->d_lut_dt, c->d_lut_s_dt, c->d_Rf, c->d_Tss, c->d_invUnl, c->d_invUop, c->d_P2, c->d_Pt,   c->d_Pr,     c->d_work,
                    c->d_flag,  c->d_scale, c->d_Er,  c->d_Ei,  c->d_A,  c->d_F32, c->d_Fb,  c->d_D,   c->d_Ptf,
                    c->d_P2s};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    free(c);
}

template <typename T>
static int dev_upload(nlse_error_slot *err, T **dst, const T *src, size_t n) {
    NLSE_CUDA_TRY(err, cudaMalloc((void **)dst, n * sizeof(T)));
    if (src) NLSE_CUDA_TRY(err, cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return NLSE_OK;
}

#define NLSE_TRY(x)                \
    do {                           \
        int s_ = (x);              \
        if (s_ != NLSE_OK) {       \
            free_ctx(c);           \
            return s_;             \
        }                          \
    } while (0)

static int check_desc(const nlse_grid_desc *d, nlse_error_slot *err) {
    if (!d) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "desc is NULL");
        return NLSE_ERR_INVALID_ARG;
    }
    if (d->Nr < 1 || d->Nr > 16384) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "Nr=%d out of range [1, 16384]", d->Nr);
        return NLSE_ERR_INVALID_ARG;
    }
    if (d->Nt < 16 || d->Nt > NLSE_MAX_NT || (d->Nt & (d->Nt - 1))) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "Nt=%d must be a power of two in [16, %d]", d->Nt,
                       NLSE_MAX_NT);
        return NLSE_ERR_INVALID_ARG;
    }
    const int full = NLSE_F_KERR_RAMAN | NLSE_F_SELF_STEEP | NLSE_F_SPACE_TIME;
    if (d->flags & ~(full | NLSE_F_STE | 0xF)) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "unknown flag bits 0x%x", d->flags & ~(full | NLSE_F_STE | 0xF));
        return NLSE_ERR_INVALID_ARG;
    }
    if (d->flags & full) {
        if (d->Nt > 4096) {
            nlse_set_error(err, NLSE_ERR_UNSUPPORTED,
                           "Raman / self-steepening / space-time focusing run the row transforms of split() in "
                           "shared memory: Nt=%d > 4096",
                           d->Nt);
            return NLSE_ERR_UNSUPPORTED;
        }
        if (((d->flags & NLSE_F_KERR_RAMAN) && !d->R_f) || ((d->flags & NLSE_F_SELF_STEEP) && !d->T_op) ||
            ((d->flags & NLSE_F_SPACE_TIME) && (!d->inv_U_nl || !d->inv_U_op)) || !(d->f_R >= 0 && d->f_R <= 1)) {
            nlse_set_error(err, NLSE_ERR_INVALID_ARG,
                           "a full-physics flag is set without its table (R_f / T_op / inv_U_nl, inv_U_op), "
                           "or f_R is outside [0, 1]");
            return NLSE_ERR_INVALID_ARG;
        }
    }
    if (d->flags & NLSE_F_STE) {
        if (d->Nt > 4096) {
            nlse_set_error(err, NLSE_ERR_UNSUPPORTED,
                           "the exciton channel's carrier march holds 11 rows of N_t floats in shared memory: "
                           "Nt=%d > 4096",
                           d->Nt);
            return NLSE_ERR_UNSUPPORTED;
        }
        if (!d->lut_s || !(d->beta_s >= 0) || !(d->inv_tau_ste >= 0) || !isfinite(d->ste_pref)) {
            nlse_set_error(err, NLSE_ERR_INVALID_ARG,
                           "NLSE_F_STE needs lut_s, beta_s >= 0, inv_tau_ste >= 0 and a finite ste_pref");
            return NLSE_ERR_INVALID_ARG;
        }
    }
    if (!d->Y || !d->rho_modes || !d->delta_k || !d->spec_mask || !d->mask_r || !d->pchip_x ||
        !d->pchip_c || !d->lut) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "a table pointer in desc is NULL");
        return NLSE_ERR_INVALID_ARG;
    }
    if (!(d->dt > 0) || !(d->komega > 0) || !(d->rho_max > 0) || !(d->invE2 > 0)) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "dt, komega, rho_max and invE2 must be positive");
        return NLSE_ERR_INVALID_ARG;
    }
    if (d->lut_n < 2) {
        nlse_set_error(err, NLSE_ERR_INVALID_ARG, "lut_n=%d < 2", d->lut_n);
        return NLSE_ERR_INVALID_ARG;
    }
    // the spline's knots must be the reference grid I = 10^d (1 + 0.01 m), d < 17, m < 900
    if (d->pchip_n != 17 * 900) {
        nlse_set_error(err, NLSE_ERR_UNSUPPORTED, "pchip_n=%d: only the 17x900 intensity grid is supported",
                       d->pchip_n);
        return NLSE_ERR_UNSUPPORTED;
    }
    for (int i = 0; i < d->pchip_n; ++i) {
        double want = pow(10.0, (double)(i / 900)) * (1.0 + 0.01 * (double)(i % 900));
        if (fabs(d->pchip_x[i] - want) > 1e-12 * want) {
            nlse_set_error(err, NLSE_ERR_UNSUPPORTED, "pchip knot %d = %g is not 10^d (1 + 0.01 m)", i,
                           d->pchip_x[i]);
            return NLSE_ERR_UNSUPPORTED;
        }
    }
    return NLSE_OK;
}

// In-place radix-2 FFT of n complex values (re, im interleaved), sign -1 forward,
// +1 inverse (unnormalised); FP64, host.
static void fft64(std::vector<double> &a, int n, int sign) {
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            std::swap(a[2 * i], a[2 * j]);
            std::swap(a[2 * i + 1], a[2 * j + 1]);
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / len;
        for (int i = 0; i < n; i += len)
            for (int k = 0; k < len / 2; ++k) {
                const double wr = cos(ang * k), wi = sin(ang * k);
                const int u = i + k, v = i + k + len / 2;
                const double xr = a[2 * v] * wr - a[2 * v + 1] * wi, xi = a[2 * v] * wi + a[2 * v + 1] * wr;
                a[2 * v] = a[2 * u] - xr;
                a[2 * v + 1] = a[2 * u + 1] - xi;
                a[2 * u] += xr;
                a[2 * u + 1] += xi;
            }
    }
}

// Whether the Raman response spectrum Rf (n complex values, the reference's
// R_f = fft(ifftshift(resp)) dt, grids.py) is a sampled damped sine, so that
// the row's circular convolution is the periodic solution of a first-order
// complex recurrence.  The kernel k = ifft(Rf) (= dt h) has k[m + 1] =
// p k[m] - q k[m - 1] with p = 2 r cos(theta), q = r^2 for such a response;
// p, q come from k[1..3] (k[0] = 0), and the recurrence's own kernel -- with
// the periodic wrap, dt h_eff[m] = Im(A z^m / (1 - z^n)), z = r e^{i theta} --
// must reproduce every k[m] to 1e-9 of its largest value (the reference's
// kernel is zero for negative times; there the recurrence's terms are below
// |z|^{n/2}).  Then *zr + i *zi = z and *amp = A.
static bool raman_fit(const double *Rf, int n, double *zr, double *zi, double *amp) {
    if (n < 8 || (n & (n - 1))) return false;
    std::vector<double> k(Rf, Rf + 2 * (size_t)n);
    fft64(k, n, +1);
    double kmax = 0.0;
    for (int m = 0; m < n; ++m) {
        k[2 * m] /= n;
        kmax = fmax(kmax, fabs(k[2 * m]));
    }
    const double k1 = k[2], k2 = k[4], k3 = k[6];
    if (!(kmax > 0.0) || !(fabs(k1) > 1e-6 * kmax)) return false;
    const double p = k2 / k1, q = (p * k2 - k3) / k1;
    if (!(q > 0.0 && q < 1.0)) return false;
    const double r = sqrt(q), c = p / (2.0 * r);
    if (!(fabs(c) < 1.0)) return false;
    const double th = acos(c), A = k1 / (r * sin(th));
    // z^n and the wrap factor 1 / (1 - z^n)
    const double rn = pow(r, (double)n), tn = th * n;
    const double wr = 1.0 - rn * cos(tn), wi = -rn * sin(tn), wd = wr * wr + wi * wi;
    double err = 0.0;
    for (int m = 0; m < n; ++m) {
        // Im(A z^m' / (1 - z^n)) with m' = m, or n for m = 0
        const int mm = m == 0 ? n : m;
        const double zm = pow(r, (double)mm), ar = A * zm * cos(th * mm), ai = A * zm * sin(th * mm);
        const double model = (ai * wr - ar * wi) / wd;
        err = fmax(err, fabs(model - k[2 * m]));
    }
    if (!(err <= 1e-9 * kmax)) return false;
    *zr = r * cos(th);
    *zi = r * sin(th);
    *amp = A;
    return true;
}

// Intensity below which lut_rate_dt's interpolation reads two zero entries of
// the W * dt table l (uniform in log10 I from log_min, inv_dlog entries per
// decade), so the rate is exactly 0: half a table interval below the point
// where the first nonzero entry starts to count.  The margin is ~1e3 times the
// FP32 error of the device's table position.  0 when the table starts nonzero;
// infinity when it is zero throughout.
static float lut_zero_below(const std::vector<float> &l, double log_min, double inv_dlog) {
    size_t k0 = 0;
    while (k0 < l.size() && l[k0] == 0.0f) ++k0;
    if (k0 >= l.size()) return INFINITY;
    if (k0 < 2) return 0.0f;
    return (float)pow(10.0, log_min + ((double)k0 - 1.5) / inv_dlog);
}

extern "C" int nlse_create(const nlse_grid_desc *d, nlse_ctx **out) {
    nlse_error_slot *gerr = &g_create_err;
    gerr->status = NLSE_OK;
    gerr->msg[0] = 0;
    if (!out) {
        nlse_set_error(gerr, NLSE_ERR_INVALID_ARG, "out is NULL");
        return NLSE_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int s = check_desc(d, gerr);
    if (s != NLSE_OK) return s;

    nlse_ctx *c = nullptr;  // 64-byte aligned: it embeds CUtensorMap objects
    if (posix_memalign((void **)&c, 64, sizeof(nlse_ctx)) == 0) memset(c, 0, sizeof(nlse_ctx));
    if (!c) {
        nlse_set_error(gerr, NLSE_ERR_INVALID_ARG, "out of host memory");
        return NLSE_ERR_INVALID_ARG;
    }
    cudaError_t ce = cudaGetDevice(&c->device);
    if (ce != cudaSuccess) {
        nlse_set_error(gerr, NLSE_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(ce));
        free(c);
        return NLSE_ERR_CUDA;
    }
    const int Nr = d->Nr, Nt = d->Nt;
    c->Nr = Nr;
    c->Nt = Nt;
    c->logNt = 0;
    while ((1 << c->logNt) < Nt) ++c->logNt;
    c->flags = d->flags;
    c->dt = d->dt;
    c->komega = d->komega;
    c->Rk_iRk = d->Rk_iRk;
    c->cached_dz = NAN;

    NLParams &nl = c->nl;
    nl.invE2 = (float)d->invE2;
    nl.kp = (d->flags & NLSE_F_KERR_INSTANT) ? (float)(d->kerr_pref * d->kerr_scale) : 0.0f;
    nl.pp_abs = (d->flags & NLSE_F_PLASMA_ABSORB) ? (float)d->plasma_pref : 0.0f;
    nl.pp_def = (d->flags & NLSE_F_PLASMA_DEFOC) ? (float)(d->plasma_pref * d->omega0_tau_c) : 0.0f;
    nl.rho_max = (float)d->rho_max;
    nl.inv_rho_max = (float)(1.0 / d->rho_max);
    nl.photo_on = (d->flags & NLSE_F_PHOTO_LOSS) ? 1 : 0;
    nl.Imin = (float)d->pchip_x[0];
    nl.Imax = (float)d->pchip_x[d->pchip_n - 1];
    nl.tiny_I = (float)(1e-30 * d->invE2);
    nl.n_int = d->pchip_n - 1;

    ScanParams &sc = c->sc;
    sc.invE2 = (float)d->invE2;
    sc.a_coef = (float)(d->beta_g * d->dt);
    sc.c_rec = (float)(d->dt * d->inv_tau_r);
    sc.na = (float)d->rho_max;
    sc.inv_na = (float)(1.0 / d->rho_max);
    sc.x_tiny = (float)(d->rho_max * 1.4901161193847656e-08);  // 2^-26
    sc.lut_log_min = (float)d->lut_log_min;
    sc.lut_inv_dlog = (float)d->lut_inv_dlog;
    sc.Imin = (float)d->lut_Imin;
    sc.Imax = (float)d->lut_Imax;
    sc.lut_n = d->lut_n;
    const bool ste = (d->flags & NLSE_F_STE) != 0;
    sc.ste = ste ? 1 : 0;
    sc.as_coef = ste ? (float)(d->beta_s * d->dt) : 0.0f;
    sc.cs_ste = ste ? (float)(d->dt * d->inv_tau_ste) : 0.0f;
    nl.ste_pref = ste ? (float)d->ste_pref : 0.0f;
    nl.kp_raman = (d->flags & NLSE_F_KERR_RAMAN) ? (float)(d->kerr_pref * d->f_R) : 0.0f;

    nlse_error_slot *err = gerr;
    // twiddles exp(-2 pi i m / Nt) in the per-pass row layout, FP64 then rounded
    {
        const int n = fft_tw_size(Nt);
        std::vector<float2> tw(n > 0 ? 2 * n : 2, make_float2(0.0f, 0.0f));
        for (int e = 0; e < n; ++e) {
            int m;
            fft_tw_entry(Nt, e, &m);
            if (m < 0) continue;
            const double a = -2.0 * M_PI * (double)m / (double)Nt, cr = cos(a), ci = sin(a);
            tw[e] = make_float2((float)cr, (float)ci);
            tw[n + e] = make_float2((float)(cr - (double)tw[e].x), (float)(ci - (double)tw[e].y));
        }
        NLSE_TRY(dev_upload(err, &c->d_tw, tw.data(), tw.size()));
    }
    {
        std::vector<float> Yf((size_t)Nr * Nr);
        for (size_t i = 0; i < Yf.size(); ++i) Yf[i] = (float)d->Y[i];
        NLSE_TRY(dev_upload(err, &c->d_Y, Yf.data(), Yf.size()));
    }
    NLSE_TRY(dev_upload(err, &c->d_rho_modes, d->rho_modes, Nr));
    NLSE_TRY(dev_upload(err, &c->d_delta_k, d->delta_k, Nt));
    NLSE_TRY(dev_upload(err, &c->d_spec_mask, d->spec_mask, Nt));
    {
        std::vector<float> m(Nr);
        for (int i = 0; i < Nr; ++i) m[i] = (float)d->mask_r[i];
        NLSE_TRY(dev_upload(err, &c->d_mask_r, m.data(), Nr));
    }
    {
        // Hermite cubic per interval in s = (I - x_i)/h_i, scaled by photo_const*invE2/x_i
        const int ni = d->pchip_n - 1;
        std::vector<float4> tab(ni);
        const double *C = d->pchip_c;
        for (int i = 0; i < ni; ++i) {
            double x = d->pchip_x[i], h = d->pchip_x[i + 1] - x;
            double sig = d->photo_const * d->invE2 / x;
            double q[4] = {C[3 * (size_t)ni + i], C[2 * (size_t)ni + i] * h, C[1 * (size_t)ni + i] * h * h,
                           C[0 * (size_t)ni + i] * h * h * h};
            float f[4];
            for (int k = 0; k < 4; ++k) {
                double v = q[k] * sig;
                if (!isfinite(v)) v = 0.0;
                if (v > FLT_MAX / 4) v = FLT_MAX / 4;
                if (v < -FLT_MAX / 4) v = -FLT_MAX / 4;
                f[k] = (float)v;
            }
            tab[i] = make_float4(f[0], f[1], f[2], f[3]);
        }
        // Below I_skip the rate is bounded by 1e-20 / m: alpha dz / 2 is then
        // far below FP32 resolution, and the kernels skip the spline there.
        // Interval i bounds the rate by the sum of its coefficients' magnitudes
        // (x_i / I <= 1 on it); below Imin the rate is |c0| Imin / (I + tiny).
        const double eps = 1e-20;
        double skip = 0.0;
        if (fabs((double)tab[0].x) * d->pchip_x[0] / (1e-30 * d->invE2) < eps) {
            skip = d->pchip_x[0];
            for (int i = 0; i < ni; ++i) {
                const double b = fabs((double)tab[i].x) + fabs((double)tab[i].y) + fabs((double)tab[i].z) +
                                 fabs((double)tab[i].w);
                if (!(b < eps)) break;
                skip = d->pchip_x[i + 1];
            }
        }
        c->nl.I_skip = (float)skip;
        NLSE_TRY(dev_upload(err, &c->d_pchip, tab.data(), ni));
    }
    {
        std::vector<float> l(d->lut_n);
        for (int k = 0; k < d->lut_n; ++k) {
            double v = d->lut[k] * d->dt;
            if (!isfinite(v) || v < 0) v = 0.0;
            if (v > FLT_MAX / 8) v = FLT_MAX / 8;
            l[k] = (float)v;
        }
        NLSE_TRY(dev_upload(err, &c->d_lut_dt, l.data(), d->lut_n));
        c->sc.I_w0 = lut_zero_below(l, d->lut_log_min, d->lut_inv_dlog);
        c->sc.I_w0s = 0.0f;
        if (d->flags & NLSE_F_STE) {
            for (int k = 0; k < d->lut_n; ++k) {
                double v = d->lut_s[k] * d->dt;
                if (!isfinite(v) || v < 0) v = 0.0;
                if (v > FLT_MAX / 8) v = FLT_MAX / 8;
                l[k] = (float)v;
            }
            NLSE_TRY(dev_upload(err, &c->d_lut_s_dt, l.data(), d->lut_n));
            c->sc.I_w0s = lut_zero_below(l, d->lut_log_min, d->lut_inv_dlog);
        }
    }
    c->full_nl = (d->flags & (NLSE_F_KERR_RAMAN | NLSE_F_SELF_STEEP | NLSE_F_SPACE_TIME)) != 0;
    if (d->flags & NLSE_F_KERR_RAMAN) {
        std::vector<float2> rf(Nt);
        for (int k = 0; k < Nt; ++k) rf[k] = make_float2((float)d->R_f[2 * k], (float)d->R_f[2 * k + 1]);
        NLSE_TRY(dev_upload(err, &c->d_Rf, rf.data(), Nt));
        double zr = 0, zi = 0, amp = 0;
        c->raman_iir = raman_fit(d->R_f, Nt, &zr, &zi, &amp) ? 1 : 0;
        c->raman_z = make_float2((float)zr, (float)zi);
        c->raman_amp = (float)amp;
    }
    if (d->flags & NLSE_F_SELF_STEEP) {
        std::vector<float> t(Nt);
        for (int k = 0; k < Nt; ++k) t[k] = (float)d->T_op[k];
        NLSE_TRY(dev_upload(err, &c->d_Tss, t.data(), Nt));
    }
    if (d->flags & NLSE_F_SPACE_TIME) {
        std::vector<float> t(Nt);
        for (int k = 0; k < Nt; ++k) t[k] = (float)d->inv_U_nl[k];
        NLSE_TRY(dev_upload(err, &c->d_invUnl, t.data(), Nt));
        NLSE_TRY(dev_upload(err, &c->d_invUop, d->inv_U_op, Nt));
        NLSE_TRY(dev_upload<float2>(err, &c->d_P2, nullptr, (size_t)Nr * Nt));
    }
    NLSE_TRY(dev_upload<float2>(err, &c->d_Pt, nullptr, Nt));
    NLSE_TRY(dev_upload<float2>(err, &c->d_Pr, nullptr, Nr));
    NLSE_TRY(dev_upload<float2>(err, &c->d_work, nullptr, (size_t)Nr * Nt));
    NLSE_TRY(dev_upload<int>(err, &c->d_flag, nullptr, 4));
    NLSE_TRY(dev_upload<int>(err, &c->d_scale, nullptr, NLSE_SC_N));
    // split (tensor-core) path: operator terms, Omega-domain state, tensor maps.
    // Each plane of the state and each block of E' has Nrp = Nr rounded up to
    // 64 rows (the product tiles 2 Nrp by 128); the padding rows and columns
    // are zero and no kernel writes them.  N_t < 256 is one partial tile
    // column: its loads read zeros past N_t and its stores stop at N_t.
    c->a_terms = 3;
    c->cached_dz_op = NAN;
    c->stf = (d->flags & NLSE_F_SPACE_TIME) != 0;
    // the space-time-focusing product is block-diagonal: each block must be whole 128-row tiles
    c->Nrp = c->stf ? (Nr + 127) / 128 * 128 : (Nr + 63) / 64 * 64;
    c->split_ok = c->Nrp <= 8192;
    c->stf = c->stf && c->split_ok;
    if (c->split_ok) {
        const size_t K2 = 2 * (size_t)c->Nrp;
        NLSE_TRY(dev_upload(err, &c->d_Y64, d->Y, (size_t)Nr * Nr));
        NLSE_TRY(dev_upload<double>(err, &c->d_Er, nullptr, (size_t)Nr * Nr));
        NLSE_TRY(dev_upload<double>(err, &c->d_Ei, nullptr, (size_t)Nr * Nr));
        NLSE_TRY(dev_upload<__nv_bfloat16>(err, &c->d_A, nullptr, 3 * K2 * K2));
        NLSE_TRY(dev_upload<float>(err, &c->d_F32, nullptr, K2 * Nt));
        NLSE_TRY(dev_upload<__nv_bfloat16>(err, &c->d_Fb, nullptr, 2 * K2 * Nt));
        NLSE_TRY(dev_upload<float>(err, &c->d_D, nullptr, K2 * Nt));
        NLSE_TRY(dev_upload<float2>(err, &c->d_Ptf, nullptr, 2 * (size_t)Nt));
        if (c->stf) NLSE_TRY(dev_upload<float4>(err, &c->d_P2s, nullptr, (size_t)Nr * Nt));
        {
            cudaError_t ze = cudaMemset(c->d_F32, 0, K2 * Nt * sizeof(float));
            if (ze == cudaSuccess) ze = cudaMemset(c->d_Fb, 0, 2 * K2 * Nt * sizeof(__nv_bfloat16));
            if (ze == cudaSuccess) ze = cudaMemset(c->d_D, 0, K2 * Nt * sizeof(float));
            if (ze != cudaSuccess) {
                nlse_set_error(err, NLSE_ERR_CUDA, "state init: %s", cudaGetErrorString(ze));
                free_ctx(c);
                return NLSE_ERR_CUDA;
            }
        }
        alignas(64) CUtensorMap m;
        cuuint32_t estr[2] = {1, 1};
        EncodeTiledFn cuTensorMapEncodeTiled = encode_tiled();
        if (!cuTensorMapEncodeTiled) {
            nlse_set_error(err, NLSE_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
            free_ctx(c);
            return NLSE_ERR_CUDA;
        }
        {
            cuuint64_t dims[2] = {K2, 3 * K2};
            cuuint64_t strides[1] = {K2 * 2};
            cuuint32_t box[2] = {64, 128};
            CUresult r = cuTensorMapEncodeTiled(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->d_A, dims, strides, box,
                                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) {
                nlse_set_error(err, NLSE_ERR_CUDA, "cuTensorMapEncodeTiled(A) failed: %d", (int)r);
                free_ctx(c);
                return NLSE_ERR_CUDA;
            }
            memcpy(&c->tmA, &m, sizeof(m));
        }
        {
            cuuint64_t dims[2] = {(cuuint64_t)Nt, 2 * K2};
            cuuint64_t strides[1] = {(cuuint64_t)Nt * 2};
            cuuint32_t box[2] = {64, 64};
            CUresult r = cuTensorMapEncodeTiled(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->d_Fb, dims, strides, box,
                                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) {
                nlse_set_error(err, NLSE_ERR_CUDA, "cuTensorMapEncodeTiled(B) failed: %d", (int)r);
                free_ctx(c);
                return NLSE_ERR_CUDA;
            }
            memcpy(&c->tmB, &m, sizeof(m));
        }
        {
            cuuint64_t dims[2] = {K2, 3 * K2};
            cuuint64_t strides[1] = {K2 * 2};
            cuuint32_t box[2] = {32, 128};
            CUresult r = cuTensorMapEncodeTiled(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->d_A, dims, strides, box,
                                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) {
                nlse_set_error(err, NLSE_ERR_CUDA, "cuTensorMapEncodeTiled(A32) failed: %d", (int)r);
                free_ctx(c);
                return NLSE_ERR_CUDA;
            }
            memcpy(&c->tmA32, &m, sizeof(m));
        }
        {
            cuuint64_t dims[2] = {(cuuint64_t)Nt, 2 * K2};
            cuuint64_t strides[1] = {(cuuint64_t)Nt * 2};
            cuuint32_t box[2] = {64, 32};
            CUresult r = cuTensorMapEncodeTiled(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->d_Fb, dims, strides, box,
                                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) {
                nlse_set_error(err, NLSE_ERR_CUDA, "cuTensorMapEncodeTiled(B32) failed: %d", (int)r);
                free_ctx(c);
                return NLSE_ERR_CUDA;
            }
            memcpy(&c->tmB32, &m, sizeof(m));
        }
    }
    ce = cudaMemset(c->d_flag, 0, 4 * sizeof(int));
    if (ce == cudaSuccess) ce = cudaMemset(c->d_scale, 0, NLSE_SC_N * sizeof(int));
    // space-time focusing in the split forms: diag(Y, Y) in 3 scaled FP16 terms
    // (dz-independent, built once) and the bound cY of |Y w| / max |w|
    if (ce == cudaSuccess && c->stf) {
        double ymax = 0.0, rmax = 0.0;
        for (int i = 0; i < Nr; ++i) {
            double rs = 0.0;
            for (int k = 0; k < Nr; ++k) {
                const double y = fabs(d->Y[(size_t)i * Nr + k]);
                rs += y;
                ymax = y > ymax ? y : ymax;
            }
            rmax = rs > rmax ? rs : rmax;
        }
        int e = 0;
        if (ymax > 0) frexp(ymax, &e);
        c->cY = (float)rmax;
        ce = launch_split_Yb16(c->d_Y64, Nr, c->Nrp, 14 - e, reinterpret_cast<__half *>(c->d_A), c->d_scale, 0);
        c->op_f16 = 1;
    }
    // the row kernels' plans for this N_t: timed once per device (synthetic rows)
    if (ce == cudaSuccess && c->split_ok)
        ce = row_plan_tune(c->logNt, Nr, c->d_tw, c->d_lut_dt, c->d_pchip, c->d_mask_r, c->nl, c->sc, c->d_Ptf,
                           c->d_scale);
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    if (ce != cudaSuccess) {
        nlse_set_error(err, NLSE_ERR_CUDA, "context init: %s", cudaGetErrorString(ce));
        free_ctx(c);
        return NLSE_ERR_CUDA;
    }
    *out = c;
    return NLSE_OK;
}

extern "C" void nlse_destroy(nlse_ctx *c) {
    if (!c) return;
    cudaDeviceSynchronize();
    free_ctx(c);
}

extern "C" int nlse_get_last_error(const nlse_ctx *c, char *buf, size_t len) {
    const nlse_error_slot *e = c ? &c->err : &g_create_err;
    if (buf && len) {
        strncpy(buf, e->msg, len - 1);
        buf[len - 1] = 0;
    }
    return e->status;
}

extern "C" const char *nlse_version(void) { return "libnlse 0.1 (sm_103a)"; }

// ---------------------------------------------------------------- helpers
static int bad(nlse_ctx *c, int status, const char *what) {
    nlse_set_error(&c->err, status, "%s", what);
    return status;
}

static int launched(nlse_ctx *c, cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        nlse_set_error(&c->err, NLSE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
        return NLSE_ERR_CUDA;
    }
    return NLSE_OK;
}

// Bracket one launch with events on its stream when profiling is on.
struct ProfScope {
    nlse_ctx *c;
    cudaStream_t st;
    int slot;
    ProfScope(nlse_ctx *c_, int kid, cudaStream_t s) : c(c_), st(s), slot(-1) {
        if (c->prof_on && c->prof_n < c->prof_cap) {
            slot = c->prof_n++;
            c->prof_kid[slot] = kid;
            cudaEventRecord(c->prof_ev[2 * slot], st);
        }
    }
    ~ProfScope() {
        if (slot >= 0) cudaEventRecord(c->prof_ev[2 * slot + 1], st);
    }
};
#define PROF(kid) ProfScope prof_scope_##__LINE__(c, (kid), st)

static int field_ok(nlse_ctx *c, const void *p, const char *name) {
    if (!p) {
        nlse_set_error(&c->err, NLSE_ERR_INVALID_ARG, "%s is NULL", name);
        return 0;
    }
    if ((uintptr_t)p % 16) {
        nlse_set_error(&c->err, NLSE_ERR_INVALID_ARG, "%s is not 16-byte aligned", name);
        return 0;
    }
    return 1;
}

static int ensure_tables(nlse_ctx *c, double dz, cudaStream_t st) {
    if (!(dz > 0) || !isfinite(dz)) return bad(c, NLSE_ERR_INVALID_ARG, "dz must be positive and finite");
    if (dz == c->cached_dz) return NLSE_OK;
    PROF(K_PHASE_TABLES);
    int s = launched(c, launch_phase_tables(c, dz, st), "phase tables");
    if (s == NLSE_OK && c->d_P2) s = launched(c, launch_phase_table_2d(c, dz, st), "2-d phase table");
    if (s == NLSE_OK && c->d_P2s)
        s = launched(c, launch_stf_table(c->d_rho_modes, c->d_invUop, c->Nr, c->Nt, dz, c->komega, c->d_P2s, st),
                     "space-time phase table");
    if (s == NLSE_OK) c->cached_dz = dz;
    return s;
}

static int half_linear_impl(nlse_ctx *c, float2 *u, double dz, const float *row_scale, cudaStream_t st) {
    int s = ensure_tables(c, dz, st);
    if (s) return s;
    const int M = c->Nr, N = 2 * c->Nt;
    {
        PROF(K_GEMM_F32);
        s = launched(c, launch_gemm_f32(c->d_Y, (const float *)u, (float *)c->d_work, M, N, M, nullptr, st),
                     "hankel gemm 1");
    }
    if (s) return s;
    {
        PROF(K_FFT_PHASE);
        s = launched(c, launch_fft_phase_ifft(c, c->d_work, st), "fft phase ifft");
    }
    if (s) return s;
    PROF(K_GEMM_F32);
    return launched(c, launch_gemm_f32(c->d_Y, (const float *)c->d_work, (float *)u, M, N, M, row_scale, st),
                    "hankel gemm 2");
}

// ---------------------------------------------------------------- split-BF16 path
static int autotune_gemm(nlse_ctx *c, cudaStream_t st);

static int split_ready(nlse_ctx *c, double dz, int f16, cudaStream_t st) {
    if (!c->split_ok)
        return bad(c, NLSE_ERR_UNSUPPORTED,
                   "the split (tensor-core) forms take Nr <= 8192 (this grid: use the plain mode)");
    int s = ensure_tables(c, dz, st);
    if (s) return s;
    if (c->stf) {
        // space-time focusing: the sandwich Y P(rho, Omega) Y, in FP16 terms whatever the split mode
        // (the operator diag(Y, Y) was built at creation; P(rho, Omega) per dz in ensure_tables)
        (void)f16;
        return autotune_gemm(c, st);
    }
    if (dz == c->cached_dz_op && f16 == c->op_f16) return NLSE_OK;
    {
        PROF(K_BUILD_OP);
        s = launched(c, launch_build_operator(c->d_Y64, c->d_rho_modes, c->Nr, c->Nrp, dz, c->komega, c->d_Er,
                                              c->d_Ei, 3, c->d_A, f16, c->d_scale, st),
                     "operator build");
    }
    if (s == NLSE_OK) {
        c->cached_dz_op = dz;
        c->op_f16 = f16;
    }
    if (s == NLSE_OK) s = autotune_gemm(c, st);
    return s;
}

static RowFusedArgs row_args(nlse_ctx *c, double dz) {
    RowFusedArgs a;
    a.Nr = c->Nr;
    a.Nt = c->Nt;
    a.logNt = c->logNt;
    a.Nrp = c->Nrp;
    a.tw = c->d_tw;
    a.Pt = c->d_Ptf;
    a.mask_r = c->d_mask_r;
    a.lut = c->d_lut_dt;
    a.pchip = c->d_pchip;
    a.nl = c->nl;
    a.sc = c->sc;
    a.dz = (float)dz;
    a.stats = c->d_flag;
    a.rho_s = nullptr;
    a.ft = FullTabs{c->d_Tss, c->d_invUnl, c->d_Rf, c->raman_z, c->raman_amp, c->raman_iir};
    a.f16 = c->op_f16;
    a.scale = c->d_scale;
    a.stf = c->stf;
    return a;
}

#define NLSE_SEQ_(x)             \
    do {                         \
        int s_ = (x);            \
        if (s_) return s_;       \
    } while (0)

static cudaError_t tc_gemm_raw(nlse_ctx *c, int variant, cudaStream_t st) {
    const int K2 = 2 * c->Nrp;
    const CUtensorMap *a = variant ? &c->tmA32 : &c->tmA, *b = variant ? &c->tmB32 : &c->tmB;
    // operator terms: 3 FP16 (space-time focusing: Y), 2 FP16 (merged E, split-FP16), or a_terms BF16
    const int terms = c->stf ? NLSE_STF_Y_TERMS : (c->op_f16 ? 2 : c->a_terms);
    return launch_gemm_tc(a, b, c->d_D, K2, c->Nt, K2, terms, variant, c->op_f16, c->stf, c->d_flag, st);
}

static int tc_gemm(nlse_ctx *c, cudaStream_t st) {
    PROF(K_GEMM_TC);
    return launched(c, tc_gemm_raw(c, c->gemm_variant, st), "tcgen05 gemm");
}

// The linear half step's product on GEMM input g: E'w (merged operator), or with
// space-time focusing Y P Y w -- product, phase pass, product.
static int linear_product(nlse_ctx *c, int g, cudaStream_t st) {
    NLSE_SEQ_(tc_gemm(c, st));
    if (!c->stf) return NLSE_OK;
    {
        PROF(K_STF_PHASE);
        NLSE_SEQ_(launched(c, launch_stf_phase(c->d_D, c->d_P2s, c->d_Fb, c->Nr, c->Nrp, c->Nt, c->cY, g, c->d_scale,
                                               st),
                           "space-time phase"));
    }
    return tc_gemm(c, st);
}

// Pipeline autotuner: time each (k depth, stages) variant of the tensor-core
// product on this context's live operands and keep the faster.  Runs once per
// context, on its first split-mode call (it synchronises the stream).
static int autotune_gemm(nlse_ctx *c, cudaStream_t st) {
    if (c->tuned) return NLSE_OK;
    cudaEvent_t e0, e1;
    NLSE_CUDA_TRY(&c->err, cudaEventCreate(&e0));
    NLSE_CUDA_TRY(&c->err, cudaEventCreate(&e1));
    // both variants once untimed, then timed in turn over three rounds; each
    // keeps its fastest round (a variant timed while the clock still ramps up
    // is not chosen for that)
    float best[2] = {1e30f, 1e30f};
    cudaError_t e = cudaSuccess;
    for (int v = 0; v < 2 && e == cudaSuccess; ++v) e = tc_gemm_raw(c, v, st);
    for (int round = 0; round < 3 && e == cudaSuccess; ++round) {
        for (int v = 0; v < 2 && e == cudaSuccess; ++v) {
            e = cudaEventRecord(e0, st);
            for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) e = tc_gemm_raw(c, v, st);
            if (e == cudaSuccess) e = cudaEventRecord(e1, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 1e30f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess && ms < best[v]) best[v] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return launched(c, e, "gemm autotune");
    const int pick = best[1] < best[0] ? 1 : 0;
    c->gemm_variant = pick;
    c->tuned = 1;
    return NLSE_OK;
}

#define NLSE_SEQ(x)              \
    do {                         \
        int s_ = (x);            \
        if (s_) return s_;       \
    } while (0)

// The entry writes GEMM input 0; in the split-FP16 form its scale comes from
// a bound of the physical field computed just before.
static int row_entry(nlse_ctx *c, const RowFusedArgs &a, const float2 *u, float *rho, int scan, cudaStream_t st) {
    if (a.f16)
        NLSE_SEQ(launched(c, launch_field_bound(u, (size_t)c->Nr * c->Nt, c->Nt, c->d_scale, st), "field bound"));
    PROF(K_ROW_ENTRY);
    return launched(c, launch_row_entry(a, u, c->d_F32, c->d_Fb, rho, scan, st), "row entry");
}

// g: the GEMM input whose product the kernel consumes (it writes input g + 1)
static int row_nl(nlse_ctx *c, const RowFusedArgs &a, const float *rho, int g, cudaStream_t st) {
    PROF(K_ROW_NL);
    if (c->full_nl)
        return launched(c, launch_row_nl_full(a, c->d_F32, c->d_Fb, c->d_D, rho, g, st), "row nonlinear");
    return launched(c, launch_row_nl(a, c->d_F32, c->d_Fb, c->d_D, rho, g, row_plan(c->logNt, 0), st),
                    "row nonlinear");
}

static int row_next(nlse_ctx *c, const RowFusedArgs &a, float *rho, float2 *u_out, int write_state, int scan,
                    int mask, int g, cudaStream_t st) {
    PROF(K_ROW_NEXT);
    return launched(c, launch_row_next(a, c->d_F32, c->d_Fb, c->d_D, rho, u_out, write_state, scan, mask, g,
                                       row_plan(c->logNt, 1), st),
                    "row next");
}


// f16: the split-FP16 form (otherwise split-BF16).  GEMM inputs are numbered
// per call: the entry writes input 0, each row_nl / row_next consumes input g
// and (when it writes the state) produces g + 1.
static int half_linear_split(nlse_ctx *c, float2 *u, double dz, int f16, cudaStream_t st) {
    NLSE_SEQ(split_ready(c, dz, f16, st));
    RowFusedArgs a = row_args(c, dz);
    NLSE_SEQ(row_entry(c, a, u, nullptr, 0, st));
    NLSE_SEQ(linear_product(c, 0, st));
    return row_next(c, a, nullptr, u, 0, 0, 0, 0, st);
}

static int step_split(nlse_ctx *c, float2 *u, const float *rho, const float *rho_s, double dz, int f16,
                      cudaStream_t st) {
    NLSE_SEQ(split_ready(c, dz, f16, st));
    RowFusedArgs a = row_args(c, dz);
    a.rho_s = c->sc.ste ? rho_s : nullptr;
    NLSE_SEQ(row_entry(c, a, u, nullptr, 0, st));
    NLSE_SEQ(linear_product(c, 0, st));
    NLSE_SEQ(row_nl(c, a, rho, 0, st));
    NLSE_SEQ(linear_product(c, 1, st));
    return row_next(c, a, nullptr, u, 0, 0, 1, 1, st);
}

static int rate_scan(nlse_ctx *c, const float2 *u, float *rho, float *rho_s, cudaStream_t st) {
    PROF(K_RATE_SCAN);
    return launched(c, launch_rate_scan(c, u, rho, rho_s, 1, st), "rate scan");
}

// With the exciton channel the two-population march runs as its own kernel
// on the physical field that row_next writes out (to the workspace between
// steps); the one-population march stays fused into the row kernels.
static int propagate_split_ste(nlse_ctx *c, float2 *u, float *rho, float *rho_s, double dz, int n,
                               cudaStream_t st) {
    RowFusedArgs a = row_args(c, dz);
    a.rho_s = rho_s;
    NLSE_SEQ(rate_scan(c, u, rho, rho_s, st));
    NLSE_SEQ(row_entry(c, a, u, nullptr, 0, st));
    for (int i = 0; i < n; ++i) {
        const bool last = i == n - 1;
        NLSE_SEQ(linear_product(c, 2 * i, st));
        NLSE_SEQ(row_nl(c, a, rho, 2 * i, st));
        NLSE_SEQ(linear_product(c, 2 * i + 1, st));
        NLSE_SEQ(row_next(c, a, nullptr, last ? u : c->d_work, last ? 0 : 1, 0, 1, 2 * i + 1, st));
        if (!last) NLSE_SEQ(rate_scan(c, c->d_work, rho, rho_s, st));
    }
    return NLSE_OK;
}

static int propagate_split(nlse_ctx *c, float2 *u, float *rho, float *rho_s, double dz, int n, int f16,
                           cudaStream_t st) {
    if (n == 0) return NLSE_OK;
    NLSE_SEQ(split_ready(c, dz, f16, st));
    if (c->sc.ste) return propagate_split_ste(c, u, rho, rho_s, dz, n, st);
    RowFusedArgs a = row_args(c, dz);
    if (rho_s)
        NLSE_SEQ(launched(c, cudaMemsetAsync(rho_s, 0, (size_t)c->Nr * c->Nt * sizeof(float), st), "rho_s memset"));
    NLSE_SEQ(row_entry(c, a, u, rho, 1, st));
    for (int i = 0; i < n; ++i) {
        const bool last = i == n - 1;
        NLSE_SEQ(linear_product(c, 2 * i, st));
        NLSE_SEQ(row_nl(c, a, rho, 2 * i, st));
        NLSE_SEQ(linear_product(c, 2 * i + 1, st));
        NLSE_SEQ(row_next(c, a, rho, last ? u : nullptr, last ? 0 : 1, last ? 0 : 1, 1, 2 * i + 1, st));
    }
    return NLSE_OK;
}

// ---------------------------------------------------------------- entry points
extern "C" int nlse_half_linear(nlse_ctx *c, void *u, double dz, void *stream) {
    return nlse_half_linear_ex(c, u, dz, NLSE_MODE_PLAIN_F32, stream);
}

extern "C" int nlse_half_linear_ex(nlse_ctx *c, void *u, double dz, int mode, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u")) return NLSE_ERR_INVALID_ARG;
    if (mode == NLSE_MODE_SPLIT_BF16 || mode == NLSE_MODE_SPLIT_F16)
        return half_linear_split(c, (float2 *)u, dz, mode == NLSE_MODE_SPLIT_F16, (cudaStream_t)stream);
    if (mode != NLSE_MODE_PLAIN_F32) return bad(c, NLSE_ERR_INVALID_ARG, "unknown mode");
    return half_linear_impl(c, (float2 *)u, dz, nullptr, (cudaStream_t)stream);
}

// rho_s as the nonlinear kernels read it: NULL when the exciton channel is off.
static const float *ste_density(const nlse_ctx *c, const float *rho_s) { return c->sc.ste ? rho_s : nullptr; }

// The exciton channel needs rho_s wherever the carriers are read or marched.
static bool ste_ok(nlse_ctx *c, const float *rho_s) {
    if (!c->sc.ste) return true;
    if (!rho_s) {
        bad(c, NLSE_ERR_INVALID_ARG, "rho_s is required with the exciton channel (NLSE_F_STE)");
        return false;
    }
    return field_ok(c, rho_s, "rho_s");
}

// alpha/2 + RK4 + alpha/2 of the plain form: elementwise for the measured
// toggles, the row-resident full-physics block otherwise.
static cudaError_t nonlinear_block(nlse_ctx *c, float2 *u, const float *rho, const float *rho_s, float dz,
                                   cudaStream_t st) {
    if (c->full_nl) return launch_nl_full(c, u, rho, ste_density(c, rho_s), dz, st);
    return launch_nonlinear_step(c, u, rho, ste_density(c, rho_s), dz, st);
}

extern "C" int nlse_split(nlse_ctx *c, const void *u, const float *rho, const float *rho_s, void *rhs, float *alpha,
                          void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho") || !field_ok(c, rhs, "rhs")) return NLSE_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_SPLIT);
    if (c->full_nl)
        return launched(c, launch_split_full(c, (const float2 *)u, rho, ste_density(c, rho_s), (float2 *)rhs, alpha,
                                             st),
                        "split");
    return launched(c, launch_split(c, (const float2 *)u, rho, ste_density(c, rho_s), (float2 *)rhs, alpha, st),
                    "split");
}

extern "C" int nlse_nonlinear_step(nlse_ctx *c, void *u, const float *rho, const float *rho_s, double dz,
                                   void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho")) return NLSE_ERR_INVALID_ARG;
    if (!(dz > 0) || !isfinite(dz)) return bad(c, NLSE_ERR_INVALID_ARG, "dz must be positive and finite");
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_NONLINEAR);
    return launched(c, nonlinear_block(c, (float2 *)u, rho, rho_s, (float)dz, st), "nonlinear step");
}

extern "C" int nlse_update_plasma(nlse_ctx *c, const void *u, float *rho, float *rho_s, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho") || !ste_ok(c, rho_s)) return NLSE_ERR_INVALID_ARG;
    return rate_scan(c, (const float2 *)u, rho, rho_s, (cudaStream_t)stream);
}

extern "C" int nlse_rate_equation(nlse_ctx *c, const void *u, float *rho, float *rho_s, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho") || !ste_ok(c, rho_s)) return NLSE_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_RATE_SCAN);
    return launched(c, launch_rate_scan(c, (const float2 *)u, rho, rho_s, 0, st), "rate scan");
}

static int step_plain(nlse_ctx *c, float2 *u, const float *rho, const float *rho_s, double dz, cudaStream_t st) {
    int s = half_linear_impl(c, u, dz, nullptr, st);
    if (s) return s;
    {
        PROF(K_NONLINEAR);
        s = launched(c, nonlinear_block(c, u, rho, rho_s, (float)dz, st), "nonlinear step");
    }
    if (s) return s;
    return half_linear_impl(c, u, dz, c->d_mask_r, st);
}

extern "C" int nlse_step(nlse_ctx *c, void *u, const float *rho, const float *rho_s, double dz, int mode,
                         void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho")) return NLSE_ERR_INVALID_ARG;
    if (c->sc.ste && rho_s && !field_ok(c, rho_s, "rho_s")) return NLSE_ERR_INVALID_ARG;
    if (mode == NLSE_MODE_SPLIT_BF16 || mode == NLSE_MODE_SPLIT_F16)
        return step_split(c, (float2 *)u, rho, rho_s, dz, mode == NLSE_MODE_SPLIT_F16, (cudaStream_t)stream);
    if (mode != NLSE_MODE_PLAIN_F32) return bad(c, NLSE_ERR_INVALID_ARG, "unknown mode");
    return step_plain(c, (float2 *)u, rho, rho_s, dz, (cudaStream_t)stream);
}

extern "C" int nlse_propagate(nlse_ctx *c, void *u, float *rho, float *rho_s, double dz, int nsteps, int mode,
                              void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho") || !ste_ok(c, rho_s)) return NLSE_ERR_INVALID_ARG;
    if (nsteps < 0) return bad(c, NLSE_ERR_INVALID_ARG, "nsteps < 0");
    cudaStream_t st = (cudaStream_t)stream;
    if (mode == NLSE_MODE_SPLIT_BF16 || mode == NLSE_MODE_SPLIT_F16)
        return propagate_split(c, (float2 *)u, rho, rho_s, dz, nsteps, mode == NLSE_MODE_SPLIT_F16, st);
    if (mode != NLSE_MODE_PLAIN_F32) return bad(c, NLSE_ERR_INVALID_ARG, "unknown mode");
    for (int i = 0; i < nsteps; ++i) {
        NLSE_SEQ(rate_scan(c, (const float2 *)u, rho, rho_s, st));
        NLSE_SEQ(step_plain(c, (float2 *)u, rho, rho_s, dz, st));
    }
    return NLSE_OK;
}

extern "C" int nlse_step_batched(nlse_ctx *c, const nlse_pulse_desc *p, int n, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (n < 0 || (n > 0 && !p)) return bad(c, NLSE_ERR_INVALID_ARG, "pulses NULL or n < 0");
    for (int i = 0; i < n; ++i) {
        int s = nlse_propagate(c, p[i].u, p[i].rho, p[i].rho_s, p[i].dz, p[i].nsteps, p[i].mode, stream);
        if (s) {
            char msg[400];
            snprintf(msg, sizeof(msg), "%.399s", c->err.msg);
            nlse_set_error(&c->err, s, "pulse %d: %s", i, msg);
            return s;
        }
    }
    return NLSE_OK;
}

extern "C" int nlse_debug_operator_product(nlse_ctx *c, const float *w, float *out, double dz, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, w, "w") || !field_ok(c, out, "out")) return NLSE_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (c->stf)
        return bad(c, NLSE_ERR_UNSUPPORTED,
                   "the operator-product diagnostic shows the merged operator E'; with space-time focusing the "
                   "half step is the sandwich Y P Y");
    NLSE_SEQ(split_ready(c, dz, 0, st));
    // w's Re / Im planes (Nr rows each) into the state's planes of Nrp rows
    const size_t plane = (size_t)c->Nr * c->Nt, pplane = (size_t)c->Nrp * c->Nt;
    for (int h = 0; h < 2; ++h)
        NLSE_SEQ(launched(c, launch_split_field(w + h * plane, c->d_Fb + h * pplane, 2 * pplane, plane, st),
                          "split field"));
    NLSE_SEQ(tc_gemm(c, st));
    for (int h = 0; h < 2; ++h)
        NLSE_SEQ(launched(c, cudaMemcpyAsync(out + h * plane, c->d_D + h * pplane, plane * sizeof(float),
                                             cudaMemcpyDeviceToDevice, st),
                          "copy"));
    return NLSE_OK;
}

extern "C" int nlse_debug_wait_timeout(nlse_ctx *c, int limit_us, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (limit_us < 1 || limit_us > 1000000) return bad(c, NLSE_ERR_INVALID_ARG, "limit_us must be in [1, 1000000]");
    return launched(c, launch_wait_probe(c->d_flag, 1000ull * (unsigned long long)limit_us, (cudaStream_t)stream),
                    "wait probe");
}

extern "C" int nlse_record(nlse_ctx *c, const void *u, const float *rho, const float *rho_s, const int *bin_of_t,
                           int nbins, double *out, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho") || !field_ok(c, out, "out")) return NLSE_ERR_INVALID_ARG;
    if (nbins < 0 || nbins > 8 || (nbins && !bin_of_t)) return bad(c, NLSE_ERR_INVALID_ARG, "nbins must be 0..8");
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_RECORD);
    return launched(c, launch_record(c, (const float2 *)u, rho, rho_s, bin_of_t, nbins, out, st), "record");
}

extern "C" int nlse_set_gemm_variant(nlse_ctx *c, int variant) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (variant < -1 || variant > 3) return bad(c, NLSE_ERR_INVALID_ARG, "variant must be -1 (autotune) or 0..3");
    c->gemm_variant = variant < 0 ? 0 : variant;
    c->tuned = variant >= 0;
    c->pinned = variant >= 0;
    return NLSE_OK;
}

extern "C" int nlse_get_gemm_variant(const nlse_ctx *c) { return c ? c->gemm_variant : -1; }

static int log2_nt(int Nt) {
    if (Nt < 16 || Nt > NLSE_MAX_NT || (Nt & (Nt - 1))) return -1;
    int l = 0;
    while ((1 << l) < Nt) ++l;
    return l;
}

extern "C" int nlse_get_row_plan(int Nt, int *nl_plan, int *next_plan) {
    const int l = log2_nt(Nt);
    if (l < 0 || !nl_plan || !next_plan) return NLSE_ERR_INVALID_ARG;
    *nl_plan = row_plan_get(l, 0);
    *next_plan = row_plan_get(l, 1);
    return NLSE_OK;
}

extern "C" int nlse_set_row_plan(int Nt, int nl_plan, int next_plan) {
    const int l = log2_nt(Nt);
    if (l < 0 || nl_plan < -1 || nl_plan > 2 || next_plan < -1 || next_plan > 1) return NLSE_ERR_INVALID_ARG;
    if (row_plan_set(l, 0, nl_plan) || row_plan_set(l, 1, next_plan)) return NLSE_ERR_CUDA;
    return NLSE_OK;
}

extern "C" int nlse_set_split_terms(nlse_ctx *c, int a_terms) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (a_terms != 2 && a_terms != 3) return bad(c, NLSE_ERR_INVALID_ARG, "a_terms must be 2 or 3");
    c->a_terms = a_terms;
    return NLSE_OK;
}

extern "C" int nlse_device_status(nlse_ctx *c, int *word) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    int h[4];
    NLSE_CUDA_TRY(&c->err, cudaMemcpy(h, c->d_flag, sizeof(h), cudaMemcpyDeviceToHost));
    int sc[NLSE_SC_N];
    NLSE_CUDA_TRY(&c->err, cudaMemcpy(sc, c->d_scale, sizeof(sc), cudaMemcpyDeviceToHost));
    if (word) *word = h[0];
    if (h[0]) {
        nlse_set_error(&c->err, NLSE_ERR_TIMEOUT, "a bounded device wait gave up (status word 0x%x)", h[0]);
        return NLSE_ERR_TIMEOUT;
    }
    if (sc[NLSE_SC_OVF]) {
        nlse_set_error(&c->err, NLSE_ERR_DEVICE_FLAG,
                       "split-FP16 form: %d row writes overflowed FP16 (the field grew more than 512-fold in a half "
                       "step); use the split-BF16 form",
                       sc[NLSE_SC_OVF]);
        return NLSE_ERR_DEVICE_FLAG;
    }
    return NLSE_OK;
}

extern "C" int nlse_scan_fallback_rows(nlse_ctx *c, int *out) {
    if (!c || !out) return NLSE_ERR_INVALID_ARG;
    int h[4];
    NLSE_CUDA_TRY(&c->err, cudaMemcpy(h, c->d_flag, sizeof(h), cudaMemcpyDeviceToHost));
    *out = h[1];
    return NLSE_OK;
}

// ---------------------------------------------------------------- profiling
extern "C" int nlse_profile_start(nlse_ctx *c, int capacity) {
    if (!c || capacity < 1) return NLSE_ERR_INVALID_ARG;
    prof_free(c);
    c->prof_ev = (cudaEvent_t *)calloc(2 * (size_t)capacity, sizeof(cudaEvent_t));
    c->prof_kid = (int *)calloc(capacity, sizeof(int));
    if (!c->prof_ev || !c->prof_kid) {
        prof_free(c);
        return bad(c, NLSE_ERR_INVALID_ARG, "out of host memory for profiling records");
    }
    c->prof_cap = capacity;
    for (int i = 0; i < 2 * capacity; ++i) NLSE_CUDA_TRY(&c->err, cudaEventCreate(&c->prof_ev[i]));
    c->prof_n = 0;
    c->prof_on = 1;
    return NLSE_OK;
}

extern "C" int nlse_profile_read(nlse_ctx *c, int *launches, double *total_ms, int nkinds, int *dropped) {
    if (!c || !launches || !total_ms || nkinds < 1) return NLSE_ERR_INVALID_ARG;
    for (int k = 0; k < nkinds; ++k) {
        launches[k] = 0;
        total_ms[k] = 0.0;
    }
    if (dropped) *dropped = 0;
    if (!c->prof_ev) return NLSE_OK;
    if (c->prof_n > 0) NLSE_CUDA_TRY(&c->err, cudaEventSynchronize(c->prof_ev[2 * c->prof_n - 1]));
    for (int i = 0; i < c->prof_n; ++i) {
        float ms = 0.0f;
        NLSE_CUDA_TRY(&c->err, cudaEventElapsedTime(&ms, c->prof_ev[2 * i], c->prof_ev[2 * i + 1]));
        int k = c->prof_kid[i];
        if (k < nkinds) {
            launches[k] += 1;
            total_ms[k] += ms;
        }
    }
    c->prof_on = 0;
    return NLSE_OK;
}

extern "C" const char *nlse_kernel_name(int kid) {
    switch (kid) {
        case K_RATE_SCAN: return "k_rate_scan";
        case K_GEMM_F32: return "k_gemm_f32";
        case K_FFT_PHASE: return "k_fft_phase_ifft";
        case K_NONLINEAR: return "k_nonlinear_step";
        case K_SPLIT: return "k_split";
        case K_PHASE_TABLES: return "k_phase_tables";
        case K_GEMM_TC: return "k_gemm_tc";
        case K_ROW_ENTRY: return "k_row_entry";
        case K_ROW_NL: return "k_row_nl";
        case K_ROW_NEXT: return "k_row_next";
        case K_BUILD_OP: return "k_build_operator";
        case K_RECORD: return "k_record";
        case K_STF_PHASE: return "k_stf_phase";
        default: return "";
    }
}

// ---------------------------------------------------------------- batches of pulses
struct nlse_batch {
    nlse_error_slot err;
    int n, a_terms;
    int f16;                 // split-FP16 form (nlse_batch_set_mode)
    int last_f16;            // form of the last upload
    // CUDA graph of three non-final z-steps (GEMM inputs g = 0..5 modulo 6:
    // the kernels use g only modulo 2 and 3), replayed for the bulk of a call
    cudaStream_t cap_stream, cap_stream2;
    cudaEvent_t cap_fork, cap_join;
    cudaGraphExec_t graph;
    int graph_key[6];        // (variant, a_terms, f16, buffer generation, row-plan generation, table
                             // generation) it was captured for
    int graph_off;           // capture failed once: launch directly
    nlse_ctx **ctx;          // one context per pulse (tables, operator, state buffers)
    BatchPulse *h_pulses;    // pinned staging of the per-pulse table
    BatchPulse *d_pulses;
    CUtensorMap *d_maps;     // 4 per pulse: A, B (k depth 64), A, B (k depth 32)
    GemmTile *d_tiles;       // the tiles of the pulses without space-time focusing, then those with it
    int ntiles;              // all tiles
    int nmain;               // tiles of the pulses without space-time focusing (the batch's form)
    int main_lane, stf_lane; // of those / of the rest: the tiles of lane 0's pulses
    int *stf_idx, nstf;      // pulses with space-time focusing (products Y P Y in FP16 terms)
    int variant_of[2];       // the grouped product's pipeline variant per form (split-BF16, split-FP16),
                             // tuned on the batch's own launch; -1 until then
    struct Class {
        int logNt, nblocks;
        int full;            // its pulses have the full-physics terms (row_nl kind 3)
        int2 *d_work;        // (index into tab / the class's calls, row) per CTA
        int split;           // work entries of lane 0 (pulses [0, lane_pulse))
        int npulse, call0;   // its pulses; their BatchCall entries start at d_calls + call0
        int pulse[NLSE_TABLE_PULSES];  // the batch's index of each
        PulseTable *tab;     // the row launches' parameter table (host; copied into each launch)
    } cls[32];
    BatchCall *h_calls;      // pinned staging of the caller's buffers per pulse, class by class
    BatchCall *d_calls;
    int tab_gen;             // bumped whenever the class tables change (a captured graph holds a copy)
    // pulses with the exciton channel: their two-population march runs as a
    // kernel of its own after row_next (its pointers are launch arguments, so
    // a change of buffers re-captures the graph: ptr_gen)
    int *ste_idx, nste;
    int ptr_gen, graph_gen;
    // two lanes (pulses [0, lane_pulse) and the rest) run as parallel branches
    // of the z-step graph, so one lane's row kernels fill the other's GEMM tail
    int lane_pulse, lane_tiles;  // lane 0's pulses / tiles (tiles are in pulse order)
    int ncls;
    int *d_flag;
    cudaEvent_t staged;      // the last upload of h_pulses has been consumed
    cudaEvent_t done;        // end of the last nlse_batch_propagate's work, on last_stream
    cudaStream_t last_stream;
    int has_done;
    double last_dz;
    void *last_ptrs[3];      // u[0], rho[0] of the last upload (cheap change check)
    int uploaded;
};

static void batch_free(nlse_batch *b) {
    if (!b) return;
    if (b->ctx)
        for (int i = 0; i < b->n; ++i) nlse_destroy(b->ctx[i]);
    free(b->ctx);
    free(b->ste_idx);
    free(b->stf_idx);
    if (b->h_pulses) cudaFreeHost(b->h_pulses);
    if (b->h_calls) cudaFreeHost(b->h_calls);
    void *ptrs[] = {b->d_pulses, b->d_calls, b->d_maps, b->d_tiles, b->d_flag};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int c = 0; c < b->ncls; ++c) {
        if (b->cls[c].d_work) cudaFree(b->cls[c].d_work);
        free(b->cls[c].tab);
    }
    if (b->staged) cudaEventDestroy(b->staged);
    if (b->done) cudaEventDestroy(b->done);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->cap_stream2) cudaStreamDestroy(b->cap_stream2);
    if (b->cap_fork) cudaEventDestroy(b->cap_fork);
    if (b->cap_join) cudaEventDestroy(b->cap_join);
    free(b);
}

// The two-population march of the exciton-channel pulses of a lane (0 or 1;
// -1: all) on the physical fields row_next left in their workspaces.
static cudaError_t batch_ste_marches(nlse_batch *b, int lane, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < b->nste && e == cudaSuccess; ++j) {
        const int i = b->ste_idx[j];
        if (lane >= 0 && (i < b->lane_pulse) != (lane == 0)) continue;
        const BatchPulse &P = b->h_pulses[i];
        // a.rho_s is the caller's writable rho_s[i] (const only for the row kernels)
        e = launch_rate_scan(b->ctx[i], P.ste_work, P.rho, const_cast<float *>(P.a.rho_s), 1, st);
    }
    return e;
}

// The first march of the exciton-channel pulses, on the input fields u.
static cudaError_t batch_ste_marches_on(nlse_batch *b, void *const *u, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < b->nste && e == cudaSuccess; ++j) {
        const int i = b->ste_idx[j];
        e = launch_rate_scan(b->ctx[i], (const float2 *)u[i], b->h_pulses[i].rho,
                             const_cast<float *>(b->h_pulses[i].a.rho_s), 1, st);
    }
    return e;
}

// The row plan of a batched row-kernel kind (1: row_nl, 2: row_next; others have one plan).
static int batch_plan(int logNt, int kind) {
    return kind == 1 ? row_plan(logNt, 0) : (kind == 2 ? row_plan(logNt, 1) : 0);
}

// The products of one half step for the pulses of a lane (0 or 1; -1: all) on
// GEMM input g: one grouped launch over the pulses in the batch's form, and
// for the pulses with space-time focusing Y P Y -- a grouped launch of their
// block-diagonal products, the phase pass of each, a second grouped launch.
static cudaError_t batch_products(nlse_batch *b, int g, int lane, cudaStream_t st) {
    nlse_ctx *c = b->ctx[0];
    const int m0 = lane == 1 ? b->main_lane : 0;
    const int mn = lane < 0 ? b->nmain : (lane == 0 ? b->main_lane : b->nmain - b->main_lane);
    cudaError_t e = cudaSuccess;
    if (mn > 0)
        e = launch_gemm_tc_grouped(b->d_maps, b->d_pulses, b->d_tiles + m0, mn, b->f16 ? 2 : b->a_terms,
                                   c->gemm_variant, b->f16, b->d_flag, st);
    const int nst = b->ntiles - b->nmain;
    const int s0 = b->nmain + (lane == 1 ? b->stf_lane : 0);
    const int sn = lane < 0 ? nst : (lane == 0 ? b->stf_lane : nst - b->stf_lane);
    if (sn <= 0 || e != cudaSuccess) return e;
    e = launch_gemm_tc_grouped(b->d_maps, b->d_pulses, b->d_tiles + s0, sn, NLSE_STF_Y_TERMS, c->gemm_variant, 1, b->d_flag, st);
    for (int j = 0; j < b->nstf && e == cudaSuccess; ++j) {
        const int i = b->stf_idx[j];
        if (lane >= 0 && (i < b->lane_pulse) != (lane == 0)) continue;
        nlse_ctx *q = b->ctx[i];
        e = launch_stf_phase(q->d_D, q->d_P2s, q->d_Fb, q->Nr, q->Nrp, q->Nt, q->cY, g, q->d_scale, st);
    }
    if (e == cudaSuccess)
        e = launch_gemm_tc_grouped(b->d_maps, b->d_pulses, b->d_tiles + s0, sn, NLSE_STF_Y_TERMS, c->gemm_variant, 1, b->d_flag,
                                   st);
    return e;
}

// The grouped product's pipeline variant for the batch's form.  The grouped
// launch over every pulse's tiles (8 x 1024 x 2048: 1024 tiles on 152 SMs) is
// another load than the first pulse's own product (128 tiles), for which its
// context was tuned, and can prefer the other variant; so the batch times both
// on its own operands, once per form, as autotune_gemm does (each once
// untimed, three interleaved rounds, each keeping its fastest).  The grouped
// launch writes only the pulses' D, which the first z-step's product rewrites
// before anything reads it.  A variant pinned on the first context stands.
static int batch_tune(nlse_batch *b, cudaStream_t st) {
    nlse_ctx *c = b->ctx[0];
    if (c->pinned) return NLSE_OK;
    int &pick = b->variant_of[b->f16 ? 1 : 0];
    if (pick < 0 && b->nmain > 0) {
        const int terms = b->f16 ? 2 : b->a_terms;
        auto run = [&](int v) {
            return launch_gemm_tc_grouped(b->d_maps, b->d_pulses, b->d_tiles, b->nmain, terms, v, b->f16, b->d_flag,
                                          st);
        };
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaError_t e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        float best[2] = {1e30f, 1e30f};
        for (int v = 0; v < 2 && e == cudaSuccess; ++v) e = run(v);
        for (int round = 0; round < 3 && e == cudaSuccess; ++round) {
            for (int v = 0; v < 2 && e == cudaSuccess; ++v) {
                e = cudaEventRecord(e0, st);
                if (e == cudaSuccess) e = run(v);
                if (e == cudaSuccess) e = cudaEventRecord(e1, st);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 1e30f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e == cudaSuccess && ms < best[v]) best[v] = ms;
            }
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (e != cudaSuccess) {
            nlse_set_error(&b->err, NLSE_ERR_CUDA, "batch gemm autotune: %s", cudaGetErrorString(e));
            return NLSE_ERR_CUDA;
        }
        pick = best[1] < best[0] ? 1 : 0;
    }
    if (pick >= 0) c->gemm_variant = pick;
    return NLSE_OK;
}

// One z-step of one lane (0 or 1; -1: all pulses) on stream st: GEMM, row_nl
// (consumes input g), GEMM, row_next (consumes g + 1; writes input g + 2 and
// marches the carriers unless last).
static cudaError_t batch_zstep(nlse_batch *b, int g, int last, int lane, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    for (int half = 0; half < 2 && e == cudaSuccess; ++half) {
        e = batch_products(b, g + half, lane, st);
        for (int k = 0; k < b->ncls && e == cudaSuccess; ++k) {
            const int w0 = lane == 1 ? b->cls[k].split : 0;
            const int nw = lane < 0 ? b->cls[k].nblocks
                                    : (lane == 0 ? b->cls[k].split : b->cls[k].nblocks - b->cls[k].split);
            const int kind = half == 1 ? 2 : (b->cls[k].full ? 3 : 1);
            if (nw > 0)
                e = launch_row_batch(kind, b->cls[k].logNt, *b->cls[k].tab, b->d_calls + b->cls[k].call0,
                                     b->cls[k].d_work + w0, nw, half == 0 ? 0 : last, g + half,
                                     batch_plan(b->cls[k].logNt, kind), st);
        }
    }
    if (e == cudaSuccess && !last) e = batch_ste_marches(b, lane, st);
    return e;
}

// The graph of three non-final z-steps for the batch's current launch
// configuration; NULL (and direct launches from then on) if capture fails.
static cudaGraphExec_t batch_graph(nlse_batch *b) {
    const int key[6] = {b->ctx[0]->gemm_variant, b->a_terms, b->f16, b->nste ? b->ptr_gen : 0,
                        row_plan_generation(), b->tab_gen};
    if (b->graph && !memcmp(key, b->graph_key, sizeof(key))) return b->graph;
    if (b->graph_off) return nullptr;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->cap_stream &&
        (cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
         cudaStreamCreateWithFlags(&b->cap_stream2, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&b->cap_fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&b->cap_join, cudaEventDisableTiming) != cudaSuccess)) {
        b->graph_off = 1;
        return nullptr;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeRelaxed);
    const bool two = b->lane_tiles > 0 && b->lane_tiles < b->ntiles;
    if (two) {
        // lane 1 forks onto the second stream and joins before the capture ends
        if (e == cudaSuccess) e = cudaEventRecord(b->cap_fork, b->cap_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->cap_stream2, b->cap_fork, 0);
        for (int j = 0; j < 3 && e == cudaSuccess; ++j) e = batch_zstep(b, 2 * j, 0, 0, b->cap_stream);
        for (int j = 0; j < 3 && e == cudaSuccess; ++j) e = batch_zstep(b, 2 * j, 0, 1, b->cap_stream2);
        if (e == cudaSuccess) e = cudaEventRecord(b->cap_join, b->cap_stream2);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->cap_stream, b->cap_join, 0);
    } else {
        for (int j = 0; j < 3 && e == cudaSuccess; ++j) e = batch_zstep(b, 2 * j, 0, -1, b->cap_stream);
    }
    cudaError_t e2 = cudaStreamEndCapture(b->cap_stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b->graph = nullptr;
        b->graph_off = 1;
        return nullptr;
    }
    memcpy(b->graph_key, key, sizeof(key));
    return b->graph;
}

extern "C" int nlse_batch_create(const nlse_grid_desc *descs, int n, nlse_batch **out) {
    nlse_error_slot *gerr = &g_create_err;
    if (!out || !descs || n < 1) {
        nlse_set_error(gerr, NLSE_ERR_INVALID_ARG, "batch: descs/out NULL or n < 1");
        return NLSE_ERR_INVALID_ARG;
    }
    *out = nullptr;
    nlse_batch *b = (nlse_batch *)calloc(1, sizeof(nlse_batch));
    if (!b) return NLSE_ERR_INVALID_ARG;
    b->n = n;
    b->a_terms = 3;
    b->variant_of[0] = b->variant_of[1] = -1;
    b->last_dz = NAN;
    b->ctx = (nlse_ctx **)calloc(n, sizeof(nlse_ctx *));
#define BATCH_FAIL(st, ...)                       \
    do {                                         \
        nlse_set_error(gerr, (st), __VA_ARGS__); \
        batch_free(b);                           \
        return (st);                             \
    } while (0)
    for (int i = 0; i < n; ++i) {
        int st = nlse_create(&descs[i], &b->ctx[i]);
        if (st != NLSE_OK) {
            char msg[400];
            snprintf(msg, sizeof(msg), "%.399s", gerr->msg);
            BATCH_FAIL(st, "pulse %d: %s", i, msg);
        }
        if (!b->ctx[i]->split_ok)
            BATCH_FAIL(NLSE_ERR_UNSUPPORTED, "pulse %d: batches run the split forms, which take Nr <= 8192", i);
    }
    std::vector<GemmTile> tiles, stf_tiles;
    std::vector<int> stf;
    std::vector<CUtensorMap> maps(4 * (size_t)n);
    int logs[32], fulls[32], nlog = 0;
    std::vector<std::vector<int2>> work(32);
    std::vector<std::vector<int>> members(32);
    std::vector<int> ste;
    for (int i = 0; i < n; ++i) {
        nlse_ctx *c = b->ctx[i];
        // pulses built from the same QDHT tables and k0 have the same operator
        // (dz is common to the batch): they read the first such pulse's copy,
        // so the grouped product streams one operator from L2 instead of many
        // (the operator's kind too: E' of the batch's form, or diag(Y, Y) with space-time focusing)
        int owner = i;
        for (int j = 0; j < i && owner == i; ++j)
            if (descs[j].Y == descs[i].Y && descs[j].rho_modes == descs[i].rho_modes && descs[j].Nr == descs[i].Nr &&
                descs[j].komega == descs[i].komega && b->ctx[j]->stf == c->stf)
                owner = j;
        nlse_ctx *oc = b->ctx[owner];
        memcpy(&maps[4 * i], &oc->tmA, sizeof(CUtensorMap));
        memcpy(&maps[4 * i + 1], &c->tmB, sizeof(CUtensorMap));
        memcpy(&maps[4 * i + 2], &oc->tmA32, sizeof(CUtensorMap));
        memcpy(&maps[4 * i + 3], &c->tmB32, sizeof(CUtensorMap));
        const int M = 2 * c->Nrp;
        for (int m0 = 0; m0 < M; m0 += 128)
            for (int n0 = 0; n0 < c->Nt; n0 += 256) (c->stf ? stf_tiles : tiles).push_back(GemmTile{i, m0, n0, 0});
        if (c->stf) stf.push_back(i);
        // row classes: one per (N_t, full-physics terms), of at most
        // NLSE_TABLE_PULSES pulses (the parameter table of a row launch)
        int k = 0;
        while (k < nlog && (logs[k] != c->logNt || fulls[k] != c->full_nl ||
                            (int)members[k].size() >= NLSE_TABLE_PULSES))
            ++k;
        if (k == nlog) {
            if (nlog == 32)
                BATCH_FAIL(NLSE_ERR_UNSUPPORTED, "batch: more than 32 row classes (time grid x physics terms, %d pulses each)",
                           NLSE_TABLE_PULSES);
            logs[nlog] = c->logNt;
            fulls[nlog++] = c->full_nl;
        }
        const int j = (int)members[k].size();
        members[k].push_back(i);
        for (int r = 0; r < c->Nr; ++r) work[k].push_back(make_int2(j, r));
        if (c->sc.ste) ste.push_back(i);
    }
    b->nste = (int)ste.size();
    if (b->nste) {
        b->ste_idx = (int *)malloc(ste.size() * sizeof(int));
        if (!b->ste_idx) BATCH_FAIL(NLSE_ERR_INVALID_ARG, "out of host memory");
        memcpy(b->ste_idx, ste.data(), ste.size() * sizeof(int));
    }
    b->nstf = (int)stf.size();
    if (b->nstf) {
        b->stf_idx = (int *)malloc(stf.size() * sizeof(int));
        if (!b->stf_idx) BATCH_FAIL(NLSE_ERR_INVALID_ARG, "out of host memory");
        memcpy(b->stf_idx, stf.data(), stf.size() * sizeof(int));
    }
    b->nmain = (int)tiles.size();
    tiles.insert(tiles.end(), stf_tiles.begin(), stf_tiles.end());
    b->ntiles = (int)tiles.size();
    // lane 0 = the first pulses up to about half of the tiles
    b->lane_pulse = 0;
    b->lane_tiles = 0;
    if (n >= 2) {
        int acc = 0, p = 0;
        while (p < n - 1 && 2 * acc < b->ntiles) {
            acc += (2 * b->ctx[p]->Nrp / 128) * ((b->ctx[p]->Nt + 255) / 256);
            ++p;
        }
        b->lane_pulse = p;
        b->lane_tiles = acc;
    }
    b->main_lane = b->stf_lane = 0;
    for (int t = 0; t < b->ntiles; ++t)
        if (tiles[t].pulse < b->lane_pulse) ++(t < b->nmain ? b->main_lane : b->stf_lane);
    cudaError_t e = cudaMalloc((void **)&b->d_tiles, tiles.size() * sizeof(GemmTile));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_tiles, tiles.data(), tiles.size() * sizeof(GemmTile), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_maps, maps.size() * sizeof(CUtensorMap));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_pulses, n * sizeof(BatchPulse));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_pulses, n * sizeof(BatchPulse));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_calls, n * sizeof(BatchCall));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_calls, n * sizeof(BatchCall));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_flag, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_flag, 0, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    b->ncls = nlog;
    for (int k = 0, call0 = 0; k < nlog && e == cudaSuccess; ++k) {
        b->cls[k].logNt = logs[k];
        b->cls[k].full = fulls[k];
        b->cls[k].nblocks = (int)work[k].size();
        b->cls[k].npulse = (int)members[k].size();
        b->cls[k].call0 = call0;
        call0 += b->cls[k].npulse;
        for (int j = 0; j < b->cls[k].npulse; ++j) b->cls[k].pulse[j] = members[k][j];
        b->cls[k].tab = (PulseTable *)calloc(1, sizeof(PulseTable));
        if (!b->cls[k].tab) e = cudaErrorMemoryAllocation;
        b->cls[k].split = 0;
        for (const int2 &w : work[k]) b->cls[k].split += members[k][w.x] < b->lane_pulse;
        e = cudaMalloc((void **)&b->cls[k].d_work, work[k].size() * sizeof(int2));
        if (e == cudaSuccess)
            e = cudaMemcpy(b->cls[k].d_work, work[k].data(), work[k].size() * sizeof(int2), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) BATCH_FAIL(NLSE_ERR_CUDA, "batch set-up: %s", cudaGetErrorString(e));
#undef BATCH_FAIL
    *out = b;
    return NLSE_OK;
}

extern "C" void nlse_batch_destroy(nlse_batch *b) {
    if (!b) return;
    cudaDeviceSynchronize();
    batch_free(b);
}

extern "C" int nlse_batch_get_context(nlse_batch *b, int i, nlse_ctx **out) {
    if (!b || !out || i < 0 || i >= b->n) return NLSE_ERR_INVALID_ARG;
    *out = b->ctx[i];
    return NLSE_OK;
}

extern "C" int nlse_batch_set_mode(nlse_batch *b, int mode) {
    if (!b || (mode != NLSE_MODE_SPLIT_BF16 && mode != NLSE_MODE_SPLIT_F16)) return NLSE_ERR_INVALID_ARG;
    b->f16 = mode == NLSE_MODE_SPLIT_F16;
    return NLSE_OK;
}

extern "C" int nlse_batch_set_split_terms(nlse_batch *b, int a_terms) {
    if (!b || (a_terms != 2 && a_terms != 3)) return NLSE_ERR_INVALID_ARG;
    b->a_terms = a_terms;
    return NLSE_OK;
}

extern "C" int nlse_batch_device_status(nlse_batch *b, int *word) {
    if (!b) return NLSE_ERR_INVALID_ARG;
    int h[4];
    NLSE_CUDA_TRY(&b->err, cudaMemcpy(h, b->d_flag, sizeof(h), cudaMemcpyDeviceToHost));
    if (word) *word = h[0];
    if (h[0]) {
        nlse_set_error(&b->err, NLSE_ERR_TIMEOUT, "a bounded device wait gave up (status word 0x%x)", h[0]);
        return NLSE_ERR_TIMEOUT;
    }
    // every pulse's own flags (its exciton march, the split-FP16 overflow count)
    for (int i = 0; i < b->n; ++i) {
        const int s = nlse_device_status(b->ctx[i], nullptr);
        if (s != NLSE_OK) {
            nlse_set_error(&b->err, s, "pulse %d: %s", i, b->ctx[i]->err.msg);
            return s;
        }
    }
    return NLSE_OK;
}

extern "C" int nlse_batch_get_last_error(const nlse_batch *b, char *buf, size_t len) {
    const nlse_error_slot *e = b ? &b->err : &g_create_err;
    if (buf && len) {
        strncpy(buf, e->msg, len - 1);
        buf[len - 1] = 0;
    }
    return e->status;
}

extern "C" int nlse_batch_propagate(nlse_batch *b, void *const *u, float *const *rho, float *const *rho_s, double dz,
                                    int nsteps, void *stream) {
    if (!b || !u || !rho) return NLSE_ERR_INVALID_ARG;
    if (nsteps < 0) {
        nlse_set_error(&b->err, NLSE_ERR_INVALID_ARG, "nsteps < 0");
        return NLSE_ERR_INVALID_ARG;
    }
    if (nsteps == 0) return NLSE_OK;
    cudaStream_t st = (cudaStream_t)stream;
    nlse_ctx *c = b->ctx[0];  // profiling records go to the first pulse's context
    // A call on another stream than the last one first waits for the last
    // call's kernels: they read the pulse table and the shared per-pulse state
    // that this call is about to rewrite.
    if (b->has_done && st != b->last_stream) NLSE_CUDA_TRY(&b->err, cudaStreamWaitEvent(st, b->done, 0));
    bool changed = !(dz == b->last_dz) || !b->uploaded || b->last_f16 != b->f16;
    for (int i = 0; i < b->n; ++i) {
        if (!field_ok(b->ctx[i], u[i], "u") || !field_ok(b->ctx[i], rho[i], "rho") ||
            !ste_ok(b->ctx[i], rho_s ? rho_s[i] : nullptr)) {
            nlse_set_error(&b->err, NLSE_ERR_INVALID_ARG, "pulse %d: %s", i, b->ctx[i]->err.msg);
            return NLSE_ERR_INVALID_ARG;
        }
        int s = split_ready(b->ctx[i], dz, b->f16, st);
        if (s) {
            nlse_set_error(&b->err, s, "pulse %d: %s", i, b->ctx[i]->err.msg);
            return s;
        }
        const float *rs_i = b->ctx[i]->sc.ste ? rho_s[i] : nullptr;
        if (b->uploaded && (b->h_pulses[i].u != (float2 *)u[i] || b->h_pulses[i].rho != rho[i] ||
                            b->h_pulses[i].a.rho_s != rs_i))
            changed = true;
    }
    // the row launches' parameter tables hold everything but the caller's buffers
    const bool tab_changed = !(dz == b->last_dz) || !b->uploaded || b->last_f16 != b->f16;
    if (changed) {
        // the previous upload must be consumed before the staging buffers are rewritten
        NLSE_CUDA_TRY(&b->err, cudaEventSynchronize(b->staged));
        for (int i = 0; i < b->n; ++i) {
            nlse_ctx *q = b->ctx[i];
            BatchPulse &P = b->h_pulses[i];
            P.a = row_args(q, dz);
            P.F32 = q->d_F32;
            P.Fb = q->d_Fb;
            P.D = q->d_D;
            P.rho = rho[i];
            P.u = (float2 *)u[i];
            P.a.rho_s = q->sc.ste ? rho_s[i] : nullptr;
            P.ste_work = q->sc.ste ? q->d_work : nullptr;
            P.M = 2 * q->Nrp;
            P.N = q->Nt;
            P.K = 2 * q->Nrp;
            P.kdiag = q->stf;
        }
        for (int k = 0; k < b->ncls; ++k)
            for (int j = 0; j < b->cls[k].npulse; ++j) {
                const BatchPulse &P = b->h_pulses[b->cls[k].pulse[j]];
                b->h_calls[b->cls[k].call0 + j] = BatchCall{P.u, P.rho, P.a.rho_s, nullptr};
                if (tab_changed) {
                    BatchPulse &E = b->cls[k].tab->p[j];
                    E = P;
                    E.u = nullptr;
                    E.rho = nullptr;
                    E.a.rho_s = nullptr;
                }
            }
        if (tab_changed) ++b->tab_gen;
        NLSE_CUDA_TRY(&b->err, cudaMemcpyAsync(b->d_pulses, b->h_pulses, b->n * sizeof(BatchPulse),
                                               cudaMemcpyHostToDevice, st));
        NLSE_CUDA_TRY(&b->err, cudaMemcpyAsync(b->d_calls, b->h_calls, b->n * sizeof(BatchCall),
                                               cudaMemcpyHostToDevice, st));
        NLSE_CUDA_TRY(&b->err, cudaEventRecord(b->staged, st));
        b->last_dz = dz;
        b->last_f16 = b->f16;
        b->uploaded = 1;
        ++b->ptr_gen;
    }
    // rho_s of a pulse without the exciton channel stays zero (its march writes none)
    if (rho_s)
        for (int i = 0; i < b->n; ++i)
            if (rho_s[i] && !b->ctx[i]->sc.ste)
                NLSE_CUDA_TRY(&b->err, cudaMemsetAsync(rho_s[i], 0,
                                                       (size_t)b->ctx[i]->Nr * b->ctx[i]->Nt * sizeof(float), st));
#define BSEQ(kid, call, what)                                                          \
    do {                                                                               \
        PROF(kid);                                                                     \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            nlse_set_error(&b->err, NLSE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
            return NLSE_ERR_CUDA;                                                      \
        }                                                                              \
    } while (0)
    for (int i = 0; i < b->n; ++i)
        if (b->f16 || b->ctx[i]->stf)
            BSEQ(K_ROW_ENTRY,
                 launch_field_bound((const float2 *)u[i], (size_t)b->ctx[i]->Nr * b->ctx[i]->Nt, b->ctx[i]->Nt,
                                    b->ctx[i]->d_scale, st),
                 "batch field bound");
    // the exciton-channel pulses' first march (the entry kernel skips theirs)
    if (b->nste) BSEQ(K_RATE_SCAN, batch_ste_marches_on(b, u, st), "batch exciton march");
    for (int k = 0; k < b->ncls; ++k)
        BSEQ(K_ROW_ENTRY,
             launch_row_batch(0, b->cls[k].logNt, *b->cls[k].tab, b->d_calls + b->cls[k].call0, b->cls[k].d_work,
                              b->cls[k].nblocks, 1, -1, 0, st),
             "batch row entry");
    {
        const int s = batch_tune(b, st);
        if (s) return s;
    }
    int it = 0;
    // the bulk of the non-final steps as graph launches of three steps each
    // (not while per-launch profiling records the individual kernels)
    if (!c->prof_on && nsteps - 1 >= 3) {
        cudaGraphExec_t gx = batch_graph(b);
        for (; gx && it + 3 <= nsteps - 1; it += 3)
            BSEQ(K_GEMM_TC, cudaGraphLaunch(gx, st), "batch graph");
    }
    for (; it < nsteps; ++it) {
        const int last = it == nsteps - 1;
        BSEQ(K_GEMM_TC, batch_products(b, 2 * it, -1, st), "batch gemm");
        for (int k = 0; k < b->ncls; ++k)
            BSEQ(K_ROW_NL,
                 launch_row_batch(b->cls[k].full ? 3 : 1, b->cls[k].logNt, *b->cls[k].tab,
                                  b->d_calls + b->cls[k].call0, b->cls[k].d_work, b->cls[k].nblocks, 0, 2 * it,
                                  batch_plan(b->cls[k].logNt, b->cls[k].full ? 3 : 1), st),
                 "batch row nonlinear");
        BSEQ(K_GEMM_TC, batch_products(b, 2 * it + 1, -1, st), "batch gemm");
        for (int k = 0; k < b->ncls; ++k)
            BSEQ(K_ROW_NEXT,
                 launch_row_batch(2, b->cls[k].logNt, *b->cls[k].tab, b->d_calls + b->cls[k].call0,
                                  b->cls[k].d_work, b->cls[k].nblocks, last, 2 * it + 1,
                                  batch_plan(b->cls[k].logNt, 2), st),
                 "batch row next");
        if (!last && b->nste) BSEQ(K_RATE_SCAN, batch_ste_marches(b, -1, st), "batch exciton march");
    }
#undef BSEQ
    NLSE_CUDA_TRY(&b->err, cudaEventRecord(b->done, st));
    b->last_stream = st;
    b->has_done = 1;
    return NLSE_OK;
}
