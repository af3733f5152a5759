// C ABI of libnlse: context creation, table preparation and the drop-in
// entry points (declared and cross-referenced to the reference in include/nlse.h).
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "nlse_internal.cuh"

static thread_local nlse_error_slot g_create_err;

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
    void *ptrs[] = {c->d_tw, c->d_Y, c->d_Y64, c->d_rho_modes, c->d_delta_k, c->d_spec_mask,
                    c->d_mask_r, c->d_pchip, c->d_lut_dt, c->d_Pt, c->d_Pr, c->d_work, c->d_flag};
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
    const int unsupported = NLSE_F_KERR_RAMAN | NLSE_F_SELF_STEEP | NLSE_F_SPACE_TIME | NLSE_F_STE;
    if (d->flags & unsupported) {
        nlse_set_error(err, NLSE_ERR_UNSUPPORTED,
                       "flags 0x%x request Raman / self-steepening / space-time focusing / STE, "
                       "which this library does not implement",
                       d->flags & unsupported);
        return NLSE_ERR_UNSUPPORTED;
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

    nlse_ctx *c = (nlse_ctx *)calloc(1, sizeof(nlse_ctx));
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
    sc.lut_log_min = (float)d->lut_log_min;
    sc.lut_inv_dlog = (float)d->lut_inv_dlog;
    sc.Imin = (float)d->lut_Imin;
    sc.Imax = (float)d->lut_Imax;
    sc.lut_n = d->lut_n;

    nlse_error_slot *err = gerr;
    // twiddles exp(-2 pi i k / Nt), FP64 then rounded
    {
        std::vector<float2> tw(Nt);
        for (int k = 0; k < Nt; ++k) {
            double a = -2.0 * M_PI * (double)k / (double)Nt;
            tw[k] = make_float2((float)cos(a), (float)sin(a));
        }
        NLSE_TRY(dev_upload(err, &c->d_tw, tw.data(), Nt));
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
    }
    NLSE_TRY(dev_upload<float2>(err, &c->d_Pt, nullptr, Nt));
    NLSE_TRY(dev_upload<float2>(err, &c->d_Pr, nullptr, Nr));
    NLSE_TRY(dev_upload<float2>(err, &c->d_work, nullptr, (size_t)Nr * Nt));
    NLSE_TRY(dev_upload<int>(err, &c->d_flag, nullptr, 4));
    ce = cudaMemset(c->d_flag, 0, 4 * sizeof(int));
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

// ---------------------------------------------------------------- entry points
extern "C" int nlse_half_linear(nlse_ctx *c, void *u, double dz, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u")) return NLSE_ERR_INVALID_ARG;
    return half_linear_impl(c, (float2 *)u, dz, nullptr, (cudaStream_t)stream);
}

extern "C" int nlse_split(nlse_ctx *c, const void *u, const float *rho, void *rhs, float *alpha, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho") || !field_ok(c, rhs, "rhs")) return NLSE_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_SPLIT);
    return launched(c, launch_split(c, (const float2 *)u, rho, (float2 *)rhs, alpha, st), "split");
}

extern "C" int nlse_nonlinear_step(nlse_ctx *c, void *u, const float *rho, double dz, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho")) return NLSE_ERR_INVALID_ARG;
    if (!(dz > 0) || !isfinite(dz)) return bad(c, NLSE_ERR_INVALID_ARG, "dz must be positive and finite");
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_NONLINEAR);
    return launched(c, launch_nonlinear_step(c, (float2 *)u, rho, (float)dz, st), "nonlinear step");
}

extern "C" int nlse_update_plasma(nlse_ctx *c, const void *u, float *rho, float *rho_s, void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho")) return NLSE_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    PROF(K_RATE_SCAN);
    return launched(c, launch_rate_scan(c, (const float2 *)u, rho, rho_s, 1, st), "rate scan");
}

static int step_plain(nlse_ctx *c, float2 *u, const float *rho, double dz, cudaStream_t st) {
    int s = half_linear_impl(c, u, dz, nullptr, st);
    if (s) return s;
    {
        PROF(K_NONLINEAR);
        s = launched(c, launch_nonlinear_step(c, u, rho, (float)dz, st), "nonlinear step");
    }
    if (s) return s;
    return half_linear_impl(c, u, dz, c->d_mask_r, st);
}

extern "C" int nlse_step(nlse_ctx *c, void *u, const float *rho, const float *rho_s, double dz, int mode,
                         void *stream) {
    (void)rho_s;
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho")) return NLSE_ERR_INVALID_ARG;
    if (mode != NLSE_MODE_PLAIN_F32) return bad(c, NLSE_ERR_UNSUPPORTED, "mode not available in this build");
    return step_plain(c, (float2 *)u, rho, dz, (cudaStream_t)stream);
}

extern "C" int nlse_propagate(nlse_ctx *c, void *u, float *rho, float *rho_s, double dz, int nsteps, int mode,
                              void *stream) {
    if (!c) return NLSE_ERR_INVALID_ARG;
    if (!field_ok(c, u, "u") || !field_ok(c, rho, "rho")) return NLSE_ERR_INVALID_ARG;
    if (nsteps < 0) return bad(c, NLSE_ERR_INVALID_ARG, "nsteps < 0");
    if (mode != NLSE_MODE_PLAIN_F32) return bad(c, NLSE_ERR_UNSUPPORTED, "mode not available in this build");
    cudaStream_t st = (cudaStream_t)stream;
    for (int i = 0; i < nsteps; ++i) {
        int s;
        {
            PROF(K_RATE_SCAN);
            s = launched(c, launch_rate_scan(c, (const float2 *)u, rho, rho_s, 1, st), "rate scan");
        }
        if (s) return s;
        s = step_plain(c, (float2 *)u, rho, dz, st);
        if (s) return s;
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
        default: return "";
    }
}
