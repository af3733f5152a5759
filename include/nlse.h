/*
 * nlse.h -- C ABI of the GB300 propagator library (libnlse.so).
 *
 * Axisymmetric split-step NLSE for femtosecond pulses in fused silica on one
 * GB300 (sm_103a).  The caller owns every field buffer (device memory, e.g.
 * torch tensors passed by data pointer); a context owns only constant tables
 * and the workspace it allocates once in nlse_create.  No entry point
 * allocates device memory after nlse_create returns.
 *
 * Layout of a field: row-major (Nr rows = radius, Nt columns = time), complex
 * single precision interleaved (re, im) -- i.e. float2 / torch.complex64.
 * Carrier densities: row-major float32 (Nr x Nt), cm^-3.
 *
 * Every function returns an nlse_status.  On failure the context keeps a
 * message, readable with nlse_get_last_error (errors of calls without a
 * context are kept per host thread).  Launches are asynchronous on the given
 * stream (a cudaStream_t passed as void*; NULL = legacy default).  A context
 * is not thread-safe; use one context per host thread.  Calls on one context
 * share its workspace: issue them on one stream, or order them with events
 * when they use different streams (a batch does this itself: a call on a new
 * stream waits for the previous call's work).
 *
 * Reference interfaces replaced (paths in omatousou/Rapport, relative to
 * ".github/deliverable (3)/sim"):
 *   nlse_create           build_grids + LinearOperator/NonlinearOperator
 *                         constructors (grids.py:29-175, operators.py:35-87)
 *   nlse_half_linear      LinearOperator.half_linear     (operators.py:47-53)
 *   nlse_split            NonlinearOperator.split        (operators.py:89-146)
 *   nlse_nonlinear_step   the alpha/2 + RK4 + alpha/2 block of
 *                         Integrator.step                 (integrator.py:140-147)
 *   nlse_update_plasma    NonlinearOperator.update_plasma + the
 *                         solve_rate_equation_kernel      (operators.py:165-183,
 *                                                          kernels.py:36-106)
 *   nlse_rate_equation    the solve_rate_equation_kernel launch alone
 *                         (marches from the given t = 0 values)
 *                                                         (kernels.py:36-106)
 *   nlse_step             Integrator.step                (integrator.py:138-149)
 *   nlse_propagate        the z loop of Integrator.propagate: nsteps x
 *                         (update_plasma, step)           (integrator.py:156-158)
 *   nlse_step_batched     that loop for several pulses on one grid (the
 *                         notebooks' sweeps over run(); filament_sim.py:59-106)
 *   nlse_destroy          (context teardown; the reference frees by GC)
 */
#ifndef NLSE_H
#define NLSE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nlse_ctx nlse_ctx;

typedef enum {
    NLSE_OK = 0,
    NLSE_ERR_INVALID_ARG = 1,   /* bad pointer, size, alignment or value   */
    NLSE_ERR_UNSUPPORTED = 2,   /* physics toggle / grid not built (yet)   */
    NLSE_ERR_CUDA = 3,          /* a CUDA runtime call or launch failed    */
    NLSE_ERR_DEVICE_FLAG = 4,   /* a kernel reported a device-side error   */
    NLSE_ERR_TIMEOUT = 5        /* a bounded device wait gave up           */
} nlse_status;

/* Physics switches (Config field names, config.py:115-170). */
enum {
    NLSE_F_KERR_INSTANT   = 1 << 0,  /* enable_kerr_instantaneous   */
    NLSE_F_PHOTO_LOSS     = 1 << 1,  /* enable_photoionization_loss */
    NLSE_F_PLASMA_DEFOC   = 1 << 2,  /* enable_plasma_defocusing    */
    NLSE_F_PLASMA_ABSORB  = 1 << 3,  /* enable_plasma_absorption    */
    NLSE_F_KERR_RAMAN     = 1 << 4,  /* enable_kerr_raman  (N_t <= 4096) */
    NLSE_F_SELF_STEEP     = 1 << 5,  /* enable_self_steepening (N_t <= 4096) */
    NLSE_F_SPACE_TIME     = 1 << 6,  /* enable_space_time_focusing (N_t <= 4096;
                                        in the split modes and in batches the
                                        half step's correction runs as
                                        Y (P(rho, Omega) - 1) Y in scaled FP16
                                        terms, whichever split mode is asked
                                        for)                       */
    NLSE_F_STE            = 1 << 7   /* enable_ste (N_t <= 4096)    */
};

/* Linear-operator arithmetic used by nlse_step. */
enum {
    NLSE_MODE_PLAIN_F32 = 0,   /* FP32 SIMT Hankel products, reference order  */
    NLSE_MODE_SPLIT_BF16 = 1,  /* tcgen05 split-BF16 merged operator (I + E):
                                  E in 3 BF16 terms, field in 2, 4 MMAs      */
    NLSE_MODE_SPLIT_F16 = 2    /* the same product with E and the field each in
                                  2 scaled FP16 terms (~22 bits), 3 MMAs      */
};

/*
 * Everything the propagator needs, computed once on the host in FP64 by the
 * caller (the Python layer's build_grids).  Pointers are HOST pointers; the
 * arrays are copied during nlse_create and may be freed afterwards.
 */
typedef struct {
    int Nr;                     /* radial points (Config.N - 1)             */
    int Nt;                     /* time points, a power of two, 16..8192    */
    int flags;                  /* NLSE_F_* bits                            */
    double dt;                  /* time step [s]                             */
    double komega;              /* k0 = n0 w0 / c [1/m]                      */
    /* linear operator (grids.py:39-73) */
    const double *Y;            /* Nr*Nr quasi-discrete Hankel matrix        */
    const double *rho_modes;    /* Nr Hankel wavenumbers rho_m [1/m]         */
    const double *delta_k;      /* Nt dispersion delta_k(Omega) [1/m]        */
    const double *spec_mask;    /* Nt spectral band mask                     */
    const double *mask_r;       /* Nr radial absorber                        */
    double Rk_iRk;              /* Rk * iRk (mathematically 1)               */
    /* nonlinear step (operators.py:60-68, 89-146) */
    double invE2;               /* |u|^2 -> I [W/cm^2]                       */
    double kerr_pref;           /* 3 chi3 w0^2 / (8 k0 c^2)                  */
    double kerr_scale;          /* (1 - f_R) with the instantaneous Kerr on  */
    double plasma_pref;         /* sigma(w0)/2 * 100                         */
    double omega0_tau_c;        /* w0 tau_c (plasma phase 1 + i w0 tau_c)    */
    double rho_max;             /* rho_nt [cm^-3]                            */
    double photo_const;         /* 1e6 Ui / (n0 c eps0)                      */
    /* PCHIP rate spline on I_k = 10^d (1 + 0.01 m) (grids.py:140-146)       */
    int pchip_n;                /* number of knots (17 * 900 = 15300)        */
    const double *pchip_x;      /* pchip_n knots                             */
    const double *pchip_c;      /* 4 x (pchip_n - 1), scipy PPoly order      */
    /* carrier-rate table (grids.py:152-161, kernels.py:14-26)               */
    int lut_n;                  /* 4096                                      */
    const double *lut;          /* W(10^logI) [cm^-3 s^-1]                   */
    double lut_log_min, lut_inv_dlog, lut_Imin, lut_Imax;
    double beta_g;              /* avalanche coefficient sigma/Ui            */
    double inv_tau_r;           /* 1/tau_r (0 = recombination off)           */
    /* self-trapped excitons (used with NLSE_F_STE; grids.py:125-137)       */
    const double *lut_s;        /* W at the exciton gap on the same grid     */
    double beta_s;              /* sigma/Us                                  */
    double inv_tau_ste;         /* 1/tau_ste (0 = no decay)                  */
    double ste_pref;            /* exciton index term of split()             */
    /* full-physics split (grids.py:79-116; used with the flags above)     */
    double f_R;                 /* Raman fraction (kerr_I weights 1-f_R, f_R) */
    const double *R_f;          /* NLSE_F_KERR_RAMAN: Raman response spectrum,
                                   Nt complex, interleaved re,im, FFT order  */
    const double *T_op;         /* NLSE_F_SELF_STEEP: T-hat(Omega), Nt       */
    const double *inv_U_nl;     /* NLSE_F_SPACE_TIME: U^-1 of split(), Nt    */
    const double *inv_U_op;     /* NLSE_F_SPACE_TIME: U^-1 of half_linear, Nt */
} nlse_grid_desc;

/* Build a context on the current CUDA device. */
int nlse_create(const nlse_grid_desc *desc, nlse_ctx **out);

/* u <- half_linear(u, dz): iRk Y F^-1[e^{i phi} mask F(Rk Y u)], in place. */
int nlse_half_linear(nlse_ctx *ctx, void *u, double dz, void *stream);

/* half_linear with an explicit arithmetic: NLSE_MODE_PLAIN_F32 (reference
 * order: two FP32 Hankel products around the FFT pair), NLSE_MODE_SPLIT_BF16
 * or NLSE_MODE_SPLIT_F16 (one tcgen05 product with the merged operator
 * Y diag(P_r) Y = I + E). */
int nlse_half_linear_ex(nlse_ctx *ctx, void *u, double dz, int mode, void *stream);

/* (rhs, alpha) <- split(u, rho, rho_s): RK right-hand side and absorption
 * rate.  rhs: complex64 Nr x Nt, alpha: float32 Nr x Nt (may be NULL);
 * rho_s may be NULL (exciton index term off). */
int nlse_split(nlse_ctx *ctx, const void *u, const float *rho, const float *rho_s,
               void *rhs, float *alpha, void *stream);

/* u <- e^{-alpha dz/2} . RK4 . e^{-alpha dz/2} (u), rho / rho_s frozen,
 * in place (rho_s may be NULL). */
int nlse_nonlinear_step(nlse_ctx *ctx, void *u, const float *rho, const float *rho_s,
                        double dz, void *stream);

/* rho[:,0] = 0, then march the carrier rate equation along t for every r.
 * With the exciton channel on, rho_s (required then) is marched with rho;
 * with it off, rho_s may be NULL and is zeroed when given. */
int nlse_update_plasma(nlse_ctx *ctx, const void *u, float *rho, float *rho_s,
                       void *stream);

/* The rate-equation kernel alone: march every row from its t = 0 values
 * (rho[:,0], and rho_s[:,0] with the exciton channel; non-finite or negative
 * starts count as 0), without update_plasma's reset of that column. */
int nlse_rate_equation(nlse_ctx *ctx, const void *u, float *rho, float *rho_s,
                       void *stream);

/* Integrator.step(dz): half-linear, nonlinear block, half-linear, mask_r;
 * u in place, rho / rho_s read (frozen; rho_s may be NULL without excitons). */
int nlse_step(nlse_ctx *ctx, void *u, const float *rho, const float *rho_s,
              double dz, int mode, void *stream);

/* nsteps iterations of the z loop of Integrator.propagate:
 * update_plasma(u, rho, rho_s) then step(dz).  On return u holds the field
 * after the last step and rho the densities of the last update (computed from
 * the field entering that step), exactly as after the reference loop. */
int nlse_propagate(nlse_ctx *ctx, void *u, float *rho, float *rho_s, double dz,
                   int nsteps, int mode, void *stream);

/* Pulses that share this context's grid and physics (e.g. an energy sweep):
 * for each pulse, nsteps iterations of (update_plasma, step) in its mode, all
 * queued on the stream in order (the context's tables and operator are shared;
 * the pulses run one after another).  For pulses on different grids, or one
 * grouped launch per kernel across pulses, use the nlse_batch_* entry points. */
typedef struct nlse_pulse_desc {
    void *u;          /* complex64 Nr x Nt */
    float *rho;       /* float32 Nr x Nt */
    float *rho_s;     /* float32 Nr x Nt, or NULL (required with NLSE_F_STE) */
    double dz;
    int nsteps;
    int mode;         /* NLSE_MODE_* */
} nlse_pulse_desc;

int nlse_step_batched(nlse_ctx *ctx, const nlse_pulse_desc *pulses, int n, void *stream);

/* Diagnostic: out = E' w for a planar FP32 field w (2Nr x Nt: Re rows then
 * Im rows) through the tcgen05 product alone, E' = [[Re E, -Im E], [Im E, Re E]]
 * with E = Y diag(e^{-i rho^2 dz / 4k0}) Y - I.  out: 2Nr x Nt FP32. */
int nlse_debug_operator_product(nlse_ctx *ctx, const float *w, float *out, double dz,
                                void *stream);

/*
 * Batches: many pulses, each with its own grid (Nr <= 8192, padded inside)
 * and tables, advanced together in the split-BF16 form: per z-step ONE
 * grouped tensor-core launch per half step over every pulse's tiles, and one
 * row-kernel launch per distinct (Nt, full-physics terms).  The batch owns one
 * context per pulse.  Pulses may carry the Raman / self-steepening terms
 * (Nt <= 4096) and the exciton channel (its two-population march runs as one
 * launch per such pulse); pulses with space-time focusing run their half
 * step's correction as Y (P(rho, Omega) - 1) Y: two grouped launches of their
 * own and one phase pass per such pulse.
 */
typedef struct nlse_batch nlse_batch;
int nlse_batch_create(const nlse_grid_desc *descs, int n, nlse_batch **out);
/* u[i], rho[i], rho_s[i]: device pointers of pulse i (rho_s may be NULL or
 * hold NULLs, except for pulses with the exciton channel); same semantics as
 * nlse_propagate for every pulse. */
int nlse_batch_propagate(nlse_batch *b, void *const *u, float *const *rho,
                         float *const *rho_s, double dz, int nsteps, void *stream);
int nlse_batch_get_context(nlse_batch *b, int i, nlse_ctx **out);
/* The batch's tensor-core form: NLSE_MODE_SPLIT_BF16 (default) or
 * NLSE_MODE_SPLIT_F16. */
int nlse_batch_set_mode(nlse_batch *b, int mode);
int nlse_batch_set_split_terms(nlse_batch *b, int a_terms);
int nlse_batch_device_status(nlse_batch *b, int *word);
int nlse_batch_get_last_error(const nlse_batch *b, char *buf, size_t len);
void nlse_batch_destroy(nlse_batch *b);

/* Tensor-core pipeline of the split mode: 0 = 64-deep k slices x 2 stages,
 * 1 = 32-deep x 4 stages, 2 = 32-deep x 3 stages, 3 = 32-deep x 2 stages
 * (2 and 3 leave shared memory for other kernels' blocks on the same SM),
 * -1 = autotune (default: the first split-mode call times 0 and 1 on the
 * live operands and keeps the faster; that call synchronises its stream, so
 * make it before any stream capture).  A batch times both variants on its own
 * grouped launch at its first call in each form (also synchronising) and uses
 * its pick, unless a variant was pinned on its first pulse's context. */
int nlse_set_gemm_variant(nlse_ctx *ctx, int variant);
int nlse_get_gemm_variant(const nlse_ctx *ctx);

/* Row-kernel plans of the split forms for N_t on the current device: for
 * the nonlinear row kernel 0 = shared-memory body, 1 = register-resident body
 * (N_t >= 512), 2 = the shared-memory body with a compact FFT (one run-time
 * pass body for both transforms); for the next-state row kernel 0 = the default body
 * (register-resident from N_t = 2048), 1 = the shared-memory body (N_t >= 2048).
 * Both plans of a kernel compute identical results.  The first context with a
 * given N_t times both on synthetic rows and keeps the faster (get returns
 * -1 before that); set pins a pick (-1: time again at the next nlse_create)
 * and applies to the next launches of every context and batch on the device.
 * No counterpart in the reference (its transforms are library FFTs). */
int nlse_get_row_plan(int Nt, int *nl_plan, int *next_plan);
int nlse_set_row_plan(int Nt, int nl_plan, int next_plan);

/* Number of BF16 terms carrying E in the split mode: 3 (default; 4 MMAs per
 * k-slice) or 2 (the plain hi/lo scheme, 3 MMAs). */
int nlse_set_split_terms(nlse_ctx *ctx, int a_terms);

/* Synchronise and read the device status word: NLSE_ERR_TIMEOUT if a kernel
 * gave up a bounded wait since nlse_create (word receives the raw bits);
 * NLSE_ERR_DEVICE_FLAG if a split-FP16 field write overflowed FP16. */
int nlse_device_status(nlse_ctx *ctx, int *word);

/* Diagnostic of the failure path: launches one kernel that waits on an
 * mbarrier nothing arrives on, bounded by limit_us microseconds (1 .. 1e6;
 * the product's own waits are bounded by 2 s), then raises bit 3 of the
 * context's status word and returns, leaving no work in flight.  Afterwards
 * nlse_device_status (and the status of a batch holding ctx) reports
 * NLSE_ERR_TIMEOUT; the context stays usable.  No counterpart in the
 * reference (its failure detection is host-side only). */
int nlse_debug_wait_timeout(nlse_ctx *ctx, int limit_us, void *stream);

/* Per-radius diagnostics of one saved plane (Integrator._record,
 * integrator.py:179-224), FP64 reductions over t into out[r][6 + nbins]:
 * sum |u|^2, max rho, max rho_s, max |u|^2, sum 2 photo |u|^2,
 * sum 2 plasma |u|^2, then per time bin sum 2 (photo + plasma) |u|^2 with
 * bin_of_t[t] in [0, nbins) or -1 (device int array; nbins <= 8).  photo and
 * plasma are NonlinearOperator.loss_rates (operators.py:148-163).  out and
 * bin_of_t are device pointers; rho_s may be NULL. */
int nlse_record(nlse_ctx *ctx, const void *u, const float *rho, const float *rho_s,
                const int *bin_of_t, int nbins, double *out, void *stream);

/* Number of (row, call) pairs the carrier scan has re-marched sequentially
 * since nlse_create (saturated or non-converging rows); synchronous read. */
int nlse_scan_fallback_rows(nlse_ctx *ctx, int *out);

/* Per-launch profiling: bracket each of the next `capacity` kernel launches
 * with CUDA events on its stream (host-side records, no device allocation). */
int nlse_profile_start(nlse_ctx *ctx, int capacity);

/* Synchronise on the last record, sum each kernel kind's launches and event
 * time (ms) into launches[kind] / total_ms[kind] for kind < nkinds, and stop
 * recording.  Kind names: nlse_kernel_name(kind) ("" for unused ids). */
int nlse_profile_read(nlse_ctx *ctx, int *launches, double *total_ms, int nkinds,
                      int *dropped);
const char *nlse_kernel_name(int kind);

/*
 * Allocation-free variant of the plain half step, for callers that cannot
 * call cudaMalloc (a host application that owns all device memory through
 * its own pool, a real-time loop that must not reach the allocator, code
 * that cannot create an nlse_ctx).  No counterpart in the reference: it is an
 * addition of this library.  It needs no context and allocates nothing:
 *   Y   device, Nr x Nr float32 row-major (the QDHT matrix),
 *   Pt  device, Nt complex64: exp(i delta_k dz/2) spec_mask Rk iRk / Nt,
 *   Pr  device, Nr complex64: exp(-i rho_m^2 dz / (4 k0)),
 *   u   device, Nr x Nt complex64, transformed in place (16-byte aligned).
 * Its intermediate field and twiddles live in a static device array of
 * 4 MiB + 201 KiB that each GPU loading the library holds until exit, so
 * Nr * Nt must not exceed 524288 (larger sizes are rejected with
 * NLSE_ERR_INVALID_ARG).  The array's address is looked up on the first call
 * on each device (make that call before any stream capture); all calls share
 * the array, so calls that overlap on the GPU race.  Errors are read with
 * nlse_get_last_error(NULL, ...).
 */
int nlse_half_linear_noalloc(const float *Y, const void *Pt, const void *Pr, void *u,
                             int Nr, int Nt, void *stream);

/* Copy the last error message of ctx (or of the last failed nlse_create when
 * ctx is NULL) into buf; returns the status of that error. */
int nlse_get_last_error(const nlse_ctx *ctx, char *buf, size_t len);

/* Free the context's tables and workspace. */
void nlse_destroy(nlse_ctx *ctx);

/* Library version string. */
const char *nlse_version(void);

#ifdef __cplusplus
}
#endif
#endif /* NLSE_H */
