// Internal declarations shared by the libnlse translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/nlse.h"

#define NLSE_MAX_NT 8192
#define NLSE_ROW_THREADS 256

// ---------------------------------------------------------------- errors
struct nlse_error_slot {
    int status;
    char msg[512];
};

void nlse_set_error(nlse_error_slot *slot, int status, const char *fmt, ...);

#define NLSE_CUDA_TRY(slot, call)                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            nlse_set_error((slot), NLSE_ERR_CUDA, "%s failed: %s (%s:%d)", #call,   \
                           cudaGetErrorString(e_), __FILE__, __LINE__);             \
            return NLSE_ERR_CUDA;                                                   \
        }                                                                           \
    } while (0)

// ---------------------------------------------------------------- parameters
// Nonlinear step constants, FP32 (derived from nlse_grid_desc in FP64).
struct NLParams {
    float invE2;        // |u|^2 -> I
    float kp;           // kerr_pref * kerr_scale (0 if instantaneous Kerr off)
    float pp_abs;       // plasma_pref if absorption on else 0
    float pp_def;       // plasma_pref * w0 tau_c if defocusing on else 0
    float rho_max;      // rho_nt
    float inv_rho_max;  // 1 / rho_max
    int photo_on;       // photo-ionisation loss on
    float Imin, Imax;   // spline clip range
    float tiny_I;       // 1e-30 * invE2 (the +1e-30 of the reference, in I units)
    int n_int;          // spline intervals
    float ste_pref;     // exciton index term: rhs += i ste_pref rho_s u
    float kp_raman;     // kerr_pref * f_R (0 if Raman off)
    float I_skip;       // below this intensity the photo-ionisation rate is < 1e-20 / m (taken as 0)
};

// Tables of the full-physics split() (device, FFT order; NULL = that term off).
struct FullTabs {
    const float *T;       // T-hat(Omega) (self-steepening)
    const float *invU;    // U^-1(Omega) of split() (space-time focusing)
    const float2 *Rf;     // Raman response spectrum R_f
    // The Raman convolution as a recurrence (riir = 1): the response R_f stands
    // for, sampled, is dt h[m] = Im(ramp z^m) for m >= 1 (a damped sine), so
    // the circular convolution dt (h * I)[n] = Im(ramp G[n]) with
    // G[n] = z (G[n - 1] + I[n - 1]), periodic (see raman_fit)
    float2 rz;
    float ramp;
    int riir;
};

// Carrier-rate scan constants.
struct ScanParams {
    float invE2;
    float a_coef;       // beta_g * dt  (a_n = a_coef * I_avg)
    float c_rec;        // dt / tau_r
    float na;           // rho_max
    float inv_na;
    float x_tiny;       // na * 2^-26: below it the depletion factor is exactly 1 in FP32
    int ste;            // self-trapped-exciton channel on
    float as_coef;      // beta_s * dt (re-ionisation by avalanche of excitons)
    float cs_ste;       // dt / tau_ste
    float lut_log_min, lut_inv_dlog, Imin, Imax;
    int lut_n;
    float I_w0, I_w0s;  // below these intensities the W * dt tables (electrons, excitons) interpolate
                        // between two zero entries: the rate is exactly 0 (0: no such range)
};

// Arguments of the fused row kernels (k_rowfused.cu).
struct RowFusedArgs {
    int Nr, Nt, logNt;
    int Nrp;              // rows of one plane (Re, Im) of the Omega-domain state: Nr rounded up to 64
    const float2 *tw;     // forward twiddles
    const float2 *Pt;     // e^{i dk dz/2} spec_mask (no 1/Nt); Pt[Nt + k]: its rounding remainder
    const float *mask_r;  // Nr
    const float *lut;     // W * dt table for the march
    const float4 *pchip;  // photo-ionisation spline
    NLParams nl;
    ScanParams sc;
    float dz;
    int *stats;
    const float *rho_s;   // exciton density for the nonlinear step (NULL: channel off)
    FullTabs ft;          // full-physics split tables (all NULL: the measured toggles)
    int f16;              // split-FP16 form: scaled FP16 field terms (see NLSE_SC_*)
    int *scale;           // the pulse's scale cells (split-FP16 form)
    int stf;              // space-time focusing in the split form: D holds E(Omega) w = Y (P - 1) Y w,
                          // scaled by 2^(sa + sv) with sv in scale[NLSE_SC_VB + g % 2]
};

// Scale cells of the split-FP16 form (int each, per pulse):
//   [0..2]  ring of row-maxima |w| (float bits) of the GEMM inputs g = 0, 1, ...
//           (input g's max goes to slot g % 3; input g + 1 picks its scale from it)
//   [3..4]  exponent sb of the field terms of input g (slot 3 + g % 2)
//   [5]     exponent sa of the operator terms
//   [6]     count of field values that overflowed FP16 (an error)
//   [7]     scratch of the operator build (max |E|)
#define NLSE_SC_MAX 0
#define NLSE_SC_SB 3
#define NLSE_SC_SA 5
#define NLSE_SC_OVF 6
#define NLSE_SC_EMAX 7
//   [8..9]  space-time focusing: exponent sv of the FP16 terms of P Y w (the
//           second product's input) of GEMM input g (slot 8 + g % 2)
#define NLSE_SC_VB 8
//   [10..12] space-time focusing: ring of the maxima of |P Y w| (float bits) of the GEMM inputs
//           (input g's goes to slot 10 + g % 3; input g + 1 takes its scale from it; input 0's
//           "previous" maximum comes from a reduction over its first product, slot 12)
#define NLSE_SC_VMAX 10
#define NLSE_SC_N 16

// One pulse of a batch, as the batched kernels see it (device memory).
struct BatchPulse {
    RowFusedArgs a;       // a.rho_s: the exciton density (channel on) or NULL
    float *F32;
    __nv_bfloat16 *Fb;
    float *D;
    float *rho;
    float2 *u;
    float2 *ste_work;     // exciton channel: row_next writes the physical field here and
                          // the two-population march runs as its own kernel (else NULL)
    int M, N, K;  // GEMM sizes: 2Nrp, Nt, 2Nrp
    int kdiag;    // block-diagonal operator (space-time focusing: Y on each plane): a tile of rows in
                  // block b takes only the K range of block b
};

// The pulses of one batched row launch (one time-grid class, at most
// NLSE_TABLE_PULSES of them), passed by value as a __grid_constant__ kernel
// parameter: the row kernels read their pulse's arguments (physics constants,
// table pointers) through the constant cache, as the single-pulse kernels
// read theirs, instead of re-reading a copy in shared memory at every use
// (those reloads took a third of k_row_nl's shared-memory wavefronts).  The
// pointers to the caller's buffers (u, rho, rho_s) change from call to call;
// they are zero here and come from the class's BatchCall array in device
// memory, so a captured graph stays valid when only they change.
#define NLSE_TABLE_PULSES 64
struct PulseTable {
    BatchPulse p[NLSE_TABLE_PULSES];
};
static_assert(sizeof(PulseTable) + 64 <= 32764, "a kernel's parameters are limited to 32764 bytes");

// The caller's buffers of one pulse for one call (device memory, indexed like PulseTable).
struct BatchCall {
    float2 *u;
    float *rho;
    const float *rho_s;  // exciton density (channel on) or NULL
    void *pad;
};

// One 128 x 256 tile of the grouped tensor-core product.
struct GemmTile {
    int pulse, m0, n0, pad;
};

// ---------------------------------------------------------------- context
struct nlse_ctx {
    nlse_error_slot err;
    int device;
    int Nr, Nt, logNt, flags;
    double dt, komega, Rk_iRk;
    float2 raman_z;        // the Raman convolution as a recurrence (FullTabs::rz, ramp, riir)
    float raman_amp;
    int raman_iir;
    NLParams nl;
    ScanParams sc;
    // device tables
    float2 *d_tw;          // Nt forward twiddles exp(-2 pi i k / Nt)
    float *d_Y;            // Nr*Nr fp32 Hankel matrix (plain path)
    double *d_Y64;         // Nr*Nr fp64 (operator builder)
    double *d_rho_modes;   // Nr
    double *d_delta_k;     // Nt
    double *d_spec_mask;   // Nt
    float *d_mask_r;       // Nr
    float4 *d_pchip;       // n_int scaled Hermite coefficients
    float *d_lut_dt;       // lut_n entries of W * dt
    float *d_lut_s_dt;     // lut_n entries of W(exciton gap) * dt
    // full-physics split (allocated only for the terms the flags request)
    int full_nl;           // Raman, self-steepening or space-time focusing on
    float *d_Tss;          // Nt T-hat
    float *d_invUnl;       // Nt U^-1 of split()
    float2 *d_Rf;          // Nt Raman spectrum
    double *d_invUop;      // Nt U^-1 of half_linear (space-time focusing)
    float2 *d_P2;          // Nr x Nt phase of half_linear with space-time focusing (per dz)
    // per-dz tables (rebuilt on the stream when dz changes)
    double cached_dz;
    float2 *d_Pt;          // Nt  exp(i dk dz/2) mask Rk iRk / Nt
    float2 *d_Pr;          // Nr  exp(-i rho^2 dz / (4 k0))
    // workspace
    float2 *d_work;        // Nr*Nt complex64
    int *d_flag;           // device status word
    // split-BF16 path (allocated when Nr % 64 == 0 and Nt % 256 == 0)
    int split_ok, a_terms;
    int stf;               // space-time focusing in the split forms: d_A holds diag(Y, Y) in 3 scaled FP16
                           // terms (built once); E(Omega) w = Y (P(rho, Omega) - 1) Y w (stf_phase between)
    float cY;              // max_m sum_k |Y_mk| (bounds |Y w| by cY max |w|)
    float4 *d_P2s;         // Nr x Nt: exp(-i rho_m^2 dz U^-1(Omega_t) / (4 k0)) - 1 and its rounding remainder
    int Nrp;               // Nr rounded up to a multiple of 64: rows of one plane of the split-form state
                           // and of one block of E' (the padding rows / columns are zero)
    int op_f16;            // format of the operator in d_A (0: 3 BF16 terms, 1: 2 scaled FP16 terms)
    int *d_scale;          // NLSE_SC_N scale cells of the split-FP16 form
    double cached_dz_op;   // dz of the operator currently in d_A
    double *d_Er, *d_Ei;   // Nr*Nr FP64 scratch of the builder
    __nv_bfloat16 *d_A;    // 3 x (2Nr x 2Nr) BF16 terms of E'
    float *d_F32;          // 2Nr x Nt planar Omega-domain state
    __nv_bfloat16 *d_Fb;   // 2 x (2Nr x Nt) BF16 hi/lo of the state
    float *d_D;            // 2Nr x Nt tensor-core product
    float2 *d_Ptf;         // 2Nt exp(i dk dz/2) mask Rk iRk (no 1/Nt), then its FP32 rounding remainder
    CUtensorMap tmA;       // A operand: d_A as [3 * 2Nr][2Nr], box 64 x 128, 128-byte swizzle
    CUtensorMap tmB;       // B operand: d_Fb as [2 * 2Nr][Nt], box 64 x 64
    CUtensorMap tmA32;     // A operand, box 32 x 128, 64-byte swizzle
    CUtensorMap tmB32;     // B operand, box 64 x 32
    int gemm_variant;      // 0 = BK 64 x 2 stages, 1 = BK 32 x 4 stages (autotuned)
    int tuned;
    int pinned;            // gemm_variant set by nlse_set_gemm_variant (no tuner overrides it)
    // per-launch event profiling (off unless nlse_profile_start was called)
    int prof_on, prof_cap, prof_n;
    cudaEvent_t *prof_ev;  // 2 * prof_cap events
    int *prof_kid;         // kernel id per record
};

// kernel ids for the profiler (names in nlse_kernel_name)
enum {
    K_RATE_SCAN = 0,
    K_GEMM_F32 = 1,
    K_FFT_PHASE = 2,
    K_NONLINEAR = 3,
    K_SPLIT = 4,
    K_PHASE_TABLES = 5,
    K_GEMM_TC = 6,
    K_ROW_ENTRY = 7,
    K_ROW_NL = 8,
    K_ROW_NEXT = 9,
    K_BUILD_OP = 10,
    K_RECORD = 11,
    K_STF_PHASE = 12,
    K_NUM_KINDS = 16
};

// ---------------------------------------------------------------- launchers
// (implemented in the k_*.cu units; all asynchronous on `stream`)
cudaError_t launch_phase_tables(nlse_ctx *c, double dz, cudaStream_t stream);
cudaError_t launch_gemm_f32(const float *A, const float *B, float *C, int M, int N, int K,
                            const float *row_scale, cudaStream_t stream);
cudaError_t launch_fft_phase_ifft(nlse_ctx *c, float2 *u, cudaStream_t stream);
cudaError_t launch_nonlinear_step(nlse_ctx *c, float2 *u, const float *rho, const float *rho_s, float dz,
                                  cudaStream_t stream);
cudaError_t launch_split(nlse_ctx *c, const float2 *u, const float *rho, const float *rho_s, float2 *rhs,
                         float *alpha, cudaStream_t stream);
cudaError_t launch_nl_full(nlse_ctx *c, float2 *u, const float *rho, const float *rho_s, float dz,
                           cudaStream_t stream);
cudaError_t launch_split_full(nlse_ctx *c, const float2 *u, const float *rho, const float *rho_s, float2 *rhs,
                              float *alpha, cudaStream_t stream);
cudaError_t launch_row_nl_full(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                               const float *rho, int g, cudaStream_t st);
cudaError_t launch_phase_table_2d(nlse_ctx *c, double dz, cudaStream_t stream);
cudaError_t launch_rate_scan(nlse_ctx *c, const float2 *u, float *rho, float *rho_s,
                             int zero_first, cudaStream_t stream);
// kdiag: block-diagonal operator (rows of block b use only K range b; M = K = 2 blocks);
// a_terms = 3 with f16: the operator in 3 scaled FP16 terms (space-time focusing)
cudaError_t launch_gemm_tc(const CUtensorMap *tmA, const CUtensorMap *tmB, float *D, int M, int N, int K,
                           int a_terms, int variant, int f16, int kdiag, int *err, cudaStream_t stream);
// Builds E in FP64 and splits it: 3 (or a_terms) BF16 terms, or with f16 two
// FP16 terms of E 2^sa (sa from max |E|, stored in scale[NLSE_SC_SA]).
// E' is laid out for Nrp >= Nr rows per block, zero beyond Nr.
cudaError_t launch_build_operator(const double *Y64, const double *rho, int Nr, int Nrp, double dz, double komega,
                                  double *Er, double *Ei, int a_terms, __nv_bfloat16 *A, int f16, int *scale,
                                  cudaStream_t stream);
// Space-time focusing in the split forms (k_stf.cu).
// diag(Y, Y) (2 Nrp x 2 Nrp, zero outside the Nr x Nr blocks) as 3 FP16 terms of Y 2^sa;
// sa is written to scale[NLSE_SC_SA].
cudaError_t launch_split_Yb16(const double *Y64, int Nr, int Nrp, int sa, __half *A, int *scale,
                              cudaStream_t stream);
// P2s[m][t] = exp(-i rho_m^2 dz invU[t] / (4 k0)) - 1 (FP64, rounded) and its remainder.
cudaError_t launch_stf_table(const double *rho, const double *invU, int Nr, int Nt, double dz, double komega,
                             float4 *P2s, cudaStream_t stream);
// Between the two products of a half step: v = D 2^-(sa + sb_g) (planes of Nrp rows), v' = P2s v,
// written as FP16 terms of v' 2^sv into Fb (the second product's input) with sv from the
// largest component of the previous input's v' (every sixth input, g % 6 == 0: of its own,
// from a reduction pass first); sv goes to scale[NLSE_SC_VB + g % 2].
cudaError_t launch_stf_phase(const float *D, const float4 *P2s, __nv_bfloat16 *Fb, int Nr, int Nrp, int Nt, float cY,
                             int g, int *scale, cudaStream_t stream);

// Failure-path probe: a bounded mbarrier wait that runs out after limit_ns and
// raises bit 3 of the status word err.
cudaError_t launch_wait_probe(int *err, unsigned long long limit_ns, cudaStream_t stream);
// Split-FP16 form, before the entry kernel: scale[NLSE_SC_MAX + 2] = a bound of
// max |F[u]| (Nt max |u|, the "previous input" of input 0), slot 0 cleared.
cudaError_t launch_field_bound(const float2 *u, size_t n, int Nt, int *scale, cudaStream_t st);

cudaError_t launch_fft_phase_ifft_tables(float2 *u, int Nr, int Nt, int logNt, const float2 *tw, const float2 *Pt,
                                         const float2 *Pr, cudaStream_t stream);
void nlse_set_thread_error(int status, const char *msg);
cudaError_t launch_record(nlse_ctx *c, const float2 *u, const float *rho, const float *rho_s, const int *bin_of_t,
                          int nbins, double *out, cudaStream_t st);
// n values of w -> hi at hi[i], lo at hi[lo_off + i] (BF16)
cudaError_t launch_split_field(const float *w, __nv_bfloat16 *hi, size_t lo_off, size_t n, cudaStream_t st);
// kind 0 = entry (flag = do_scan), 1 = nonlinear, 2 = next (flag = last step of the call),
// 3 = nonlinear with the full-physics block (N_t <= 4096);
// g = index of the GEMM input the kernel consumes (the split-FP16 scales; -1 for the entry);
// plan = the row plan of kinds 1 and 2 (see row_plan); work[b] = (index into T and calls, row)
cudaError_t launch_row_batch(int kind, int logNt, const PulseTable &T, const BatchCall *calls, const int2 *work,
                             int nblocks, int flag, int g, int plan, cudaStream_t st);
cudaError_t launch_gemm_tc_grouped(const CUtensorMap *maps, const BatchPulse *P, const GemmTile *tiles, int ntiles,
                                   int a_terms, int variant, int f16, int *err, cudaStream_t stream);
cudaError_t launch_row_entry(const RowFusedArgs &a, const float2 *u, float *F32, __nv_bfloat16 *Fb, float *rho,
                             int do_scan, cudaStream_t st);
// g: index of the GEMM input whose product D the kernel consumes; it writes input g + 1;
// plan: the row plan (0 or 1; both give identical results, see row_plan)
cudaError_t launch_row_nl(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, const float *rho,
                          int g, int plan, cudaStream_t st);
cudaError_t launch_row_next(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, float *rho,
                            float2 *u_out, int write_state, int do_scan, int apply_mask, int g, int plan,
                            cudaStream_t st);
// Row plans of this device for N_t = 2^logNt: the pick of row_nl (kind 0) and
// row_next (kind 1), timed once per device and N_t on synthetic rows the first
// time a context of that N_t needs them (row_plan_tune, in nlse_create).
int row_plan(int logNt, int kind);
// Times both plans of each kind on R <= Nr synthetic rows (scratch allocated
// and freed here; Pt_scratch: 2 N_t float2 it may overwrite) unless already
// tuned for this device and N_t; synchronous.
cudaError_t row_plan_tune(int logNt, int Nr, const float2 *tw, const float *lut, const float4 *pchip,
                          const float *mask_r, const NLParams &nl, const ScanParams &sc, float2 *Pt_scratch,
                          int *scale);
int row_plan_get(int logNt, int kind);             // -1: not tuned yet
int row_plan_set(int logNt, int kind, int plan);   // plan -1: tune again at the next context creation
int row_plan_generation();                         // bumped by every row_plan_set

// ---------------------------------------------------------------- complex
__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// x (ph + pl) folding the remainder pl = p - ph of a rounded factor into the
// products before their last rounding: the factor table's own rounding no
// longer biases the result (what remains are roundings of data-dependent
// values); 8 operations instead of c_mul's 4.
__device__ __forceinline__ float2 c_mul_comp(float2 x, float2 ph, float2 pl) {
    return make_float2(fmaf(x.x, ph.x, fmaf(-x.y, ph.y, fmaf(x.x, pl.x, -x.y * pl.y))),
                       fmaf(x.x, ph.y, fmaf(x.y, ph.x, fmaf(x.x, pl.y, x.y * pl.x))));
}

// x (ph + pl) for a factor p held as its FP32 value ph and remainder pl = p - ph:
// both products of each component are formed with their exact rounding errors
// (fmaf) and summed with the remainder terms before the one final rounding, so
// the result is the nearly correctly rounded x p.  A factor table applied every
// z-step then adds no systematic error of its own (a plain product with the
// rounded ph would repeat the same relative error every step).
__device__ __forceinline__ float2 c_mul_exact(float2 x, float2 ph, float2 pl) {
    const float a = x.x * ph.x, b = x.y * ph.y, c = x.x * ph.y, d = x.y * ph.x;
    const float ea = fmaf(x.x, ph.x, -a), eb = fmaf(x.y, ph.y, -b);
    const float ec = fmaf(x.x, ph.y, -c), ed = fmaf(x.y, ph.x, -d);
    const float re = a - b, im = c + d;
    // two-sum errors of re and im
    const float bre = re - a, ere = (a - (re - bre)) + (-b - bre);
    const float bim = im - c, eim = (c - (im - bim)) + (d - bim);
    const float cre = fmaf(x.x, pl.x, -x.y * pl.y) + (ea - eb) + ere;
    const float cim = fmaf(x.x, pl.y, x.y * pl.x) + (ec + ed) + eim;
    return make_float2(re + cre, im + cim);
}

// multiply by the quarter-turn exp(-+ i pi/2): forward (-i), inverse (+i)
template <bool INV>
__device__ __forceinline__ float2 c_quarter(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// x / sqrt(2) with the constant's FP32 rounding remainder folded in before the
// one rounding (the plain product would bias every radix-8 pass the same way).
__device__ __forceinline__ float mul_rsqrt2(float x) {
    return fmaf(x, 0.70710676908493041992f, x * 1.2101617104e-08f);
}

// ---------------------------------------------------------------- small DFTs
// Decimation-in-frequency butterflies with natural-order outputs:
// V[k] = sum_r v[r] exp(-+ 2 pi i r k / R).
template <bool INV>
__device__ __forceinline__ void dft2(float2 *v) {
    float2 a = v[0];
    v[0] = c_add(a, v[1]);
    v[1] = c_sub(a, v[1]);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2 *v) {
    float2 y0 = c_add(v[0], v[2]), y1 = c_sub(v[0], v[2]);
    float2 y2 = c_add(v[1], v[3]), y3 = c_quarter<INV>(c_sub(v[1], v[3]));
    v[0] = c_add(y0, y2);
    v[2] = c_sub(y0, y2);
    v[1] = c_add(y1, y3);
    v[3] = c_sub(y1, y3);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2 *v) {
    float2 a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        a[r] = c_add(v[r], v[r + 4]);
        b[r] = c_sub(v[r], v[r + 4]);
    }
    // b_r *= w8^r, w8 = exp(-+ i pi / 4)
    b[1] = INV ? make_float2(mul_rsqrt2(b[1].x - b[1].y), mul_rsqrt2(b[1].x + b[1].y))
               : make_float2(mul_rsqrt2(b[1].x + b[1].y), mul_rsqrt2(b[1].y - b[1].x));
    b[2] = c_quarter<INV>(b[2]);
    b[3] = INV ? make_float2(-mul_rsqrt2(b[3].x + b[3].y), mul_rsqrt2(b[3].x - b[3].y))
               : make_float2(mul_rsqrt2(b[3].y - b[3].x), -mul_rsqrt2(b[3].x + b[3].y));
    dft4<INV>(a);
    dft4<INV>(b);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        v[2 * m] = a[m];
        v[2 * m + 1] = b[m];
    }
}

template <int R, bool INV>
__device__ __forceinline__ void dft_small(float2 *v) {
    if (R == 2) dft2<INV>(v);
    else if (R == 4) dft4<INV>(v);
    else dft8<INV>(v);
}

// Padded shared-memory index of a row held as float2: one pad slot per 16
// points makes every Stockham pass (loads and the strided stores) within
// 1.12x of conflict-free for 64-bit accesses (unpadded: 8-way on the first
// pass).  A row of N points occupies fft_slots(N) float2.
__host__ __device__ __forceinline__ constexpr int pidx(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ constexpr int fft_slots(int n) { return n + (n >> 4); }

// A Stockham pass's gathers and scatters as compile-time offsets from one
// padded base.  Sources j + r nb with nb = N / R a multiple of 16:
// pidx(j + r nb) = pidx(j) + r (nb + nb / 16).  Destinations d0 + r NS,
// d0 = (j - k) R + k: for NS a multiple of 16 the same; for NS = 8, d0 % 16 = k
// < 8 ((j - k) R is a multiple of 16), so d0 % 16 + 8 r crosses r / 2 extra
// 16-blocks: + 8 r + r / 2; for NS = 1 (d0 = j R, R dividing 16),
// d0 % 16 + r < 16: + r.  Other strides keep pidx per point.
__host__ __device__ constexpr bool pass_src_linear(int nb) { return nb % 16 == 0; }
__host__ __device__ constexpr bool pass_dst_linear(int NS, int R) {
    return NS % 16 == 0 || NS == 8 || (NS == 1 && 16 % R == 0);
}
__host__ __device__ constexpr int pass_dst_step(int NS, int r) {
    return NS % 16 == 0 ? r * (NS + NS / 16) : (NS == 8 ? 8 * r + (r >> 1) : r);
}

// Radix of the Stockham pass at NS (the product of the radices applied so far)
// for an N-point row: 8 while it divides what remains, then 4 or 2.
__host__ __device__ constexpr int fft_radix(int N, int NS) {
    return (N / NS) % 8 == 0 ? 8 : ((N / NS) % 4 == 0 ? 4 : 2);
}

// Twiddle table layout: the pass at NS > 1 (radix R) owns a block of
// NS * fft_tw_row(R) float2: for butterfly row k = 0 .. NS-1 the factors
// exp(-2 pi i r k (N / (NS R)) / N), r = 1 .. R-1 (padded to an even count),
// in pairs (r = 2q + 1, 2q + 2) of one float4 each, stored column-major --
// float4 q of row k at q NS + k.  The 32 lanes of a warp hold consecutive
// butterflies, i.e. consecutive k, so each 16-byte twiddle load of a warp is
// one contiguous 512-byte run (4 cache lines) instead of 32 rows spread over
// up to 2 KB; the values are those of a plain exp(-2 pi i m / N) table.
__host__ __device__ constexpr int fft_tw_row(int R) { return R == 2 ? 2 : R; }

__host__ __device__ constexpr int fft_tw_offset(int N, int NS) {
    int off = 0;
    for (int s = 1; s < NS; s *= fft_radix(N, s))
        if (s > 1) off += s * fft_tw_row(fft_radix(N, s));
    return off;
}

// float2 entries of the whole table of an N-point row (the table is followed
// by as many entries of its FP32 rounding remainders).
__host__ __device__ constexpr int fft_tw_size(int N) { return fft_tw_offset(N, N); }

// Twiddle and spectral-phase products with the tables' rounding remainders
// folded in (c_mul_comp; 2: the nearly correctly rounded c_mul_exact; 0: plain
// products).  Over 4000 z-steps the plain products' fixed rounding of each
// table entry adds up coherently to ~3e-4 of the field.
#ifndef NLSE_COMP_TWIDDLE
#define NLSE_COMP_TWIDDLE 1
#endif

// Twiddle products of butterfly k of the pass at NS (radix R) of an N-point
// row: v[r] *= exp(-+ 2 pi i r k (N / (NS R)) / N), r = 1 .. R-1, from table
// row k of the pass (and its rounding remainders).  COMP = false: plain
// products with the FP32 table, for a transform whose output is not carried
// from z-step to z-step (its fixed rounding then does not add up).
template <int R, bool INV, int N, int NS, bool COMP = true>
__device__ __forceinline__ void apply_twiddles(float2 *v, int k, const float2 *__restrict__ tw) {
    const float4 *w4 = reinterpret_cast<const float4 *>(tw + fft_tw_offset(N, NS)) + k;
    float2 w[fft_tw_row(R)];
#pragma unroll
    for (int q = 0; q < fft_tw_row(R) / 2; ++q) {
        const float4 p = __ldg(&w4[q * NS]);
        w[2 * q] = make_float2(p.x, p.y);
        w[2 * q + 1] = make_float2(p.z, p.w);
    }
    if constexpr (!COMP || !NLSE_COMP_TWIDDLE) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
            float2 x = w[r - 1];
            if (INV) x.y = -x.y;
            v[r] = c_mul(v[r], x);
        }
        return;
    }
#if NLSE_COMP_TWIDDLE
    // the table's rounding remainders follow the table
    const float4 *l4 = w4 + fft_tw_size(N) / 2;
    float2 wl[fft_tw_row(R)];
#pragma unroll
    for (int q = 0; q < fft_tw_row(R) / 2; ++q) {
        const float4 p = __ldg(&l4[q * NS]);
        wl[2 * q] = make_float2(p.x, p.y);
        wl[2 * q + 1] = make_float2(p.z, p.w);
    }
#pragma unroll
    for (int r = 1; r < R; ++r) {
        float2 x = w[r - 1], xl = wl[r - 1];
        if (INV) {
            x.y = -x.y;
            xl.y = -xl.y;
        }
#if NLSE_COMP_TWIDDLE == 2
        v[r] = c_mul_exact(v[r], x, xl);
#else
        v[r] = c_mul_comp(v[r], x, xl);
#endif
    }
#else
#pragma unroll
    for (int r = 1; r < R; ++r) {
        float2 x = w[r - 1];
        if (INV) x.y = -x.y;
        v[r] = c_mul(v[r], x);
    }
#endif
}

// One Stockham autosort pass of radix R over a row of N points (compile-time
// sizes): reads src, writes dst (padded indexing).  NS = product of the
// radices already applied; tw = the twiddle table above.
template <int R, bool INV, int N, int NS, int T, bool COMP = true>
__device__ __forceinline__ void stockham_pass(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                              const float2 *__restrict__ tw) {
    constexpr int nb = N / R;
#pragma unroll
    for (int jj = 0; jj < (nb + T - 1) / T; ++jj) {
        const int j = (int)threadIdx.x + jj * T;
        if (nb % T == 0 || j < nb) {
            const int k = j & (NS - 1);
            float2 v[R];
            if constexpr (pass_src_linear(nb)) {
                const float2 *s = src + pidx(j);
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = s[r * (nb + nb / 16)];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = src[pidx(j + r * nb)];
            }
            if (NS > 1) apply_twiddles<R, INV, N, NS, COMP>(v, k, tw);
            dft_small<R, INV>(v);
            const int d0 = (j - k) * R + k;
            if constexpr (pass_dst_linear(NS, R)) {
                float2 *d = dst + pidx(d0);
#pragma unroll
                for (int r = 0; r < R; ++r) d[pass_dst_step(NS, r)] = v[r];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) dst[pidx(d0 + r * NS)] = v[r];
            }
        }
    }
}

// Remaining passes from NS on.
template <int N, int NS, bool INV, int T, bool COMP = true>
__device__ __forceinline__ float2 *fft_passes(float2 *src, float2 *dst, const float2 *__restrict__ tw) {
    if constexpr (NS >= N) {
        return src;
    } else {
        constexpr int R = fft_radix(N, NS);
        stockham_pass<R, INV, N, NS, T, COMP>(src, dst, tw);
        __syncthreads();
        return fft_passes<N, NS * R, INV, T, COMP>(dst, src, tw);
    }
}

// Full in-CTA FFT of one row of N points (power of two, 16..8192) held in
// buf0 (padded indexing), buf1 = scratch of the same size; returns the buffer
// holding the unnormalised result.  Every thread of the CTA (T of them) calls it.
template <int N, bool INV, int T = NLSE_ROW_THREADS, bool COMP = true>
__device__ __forceinline__ float2 *fft_row(float2 *buf0, float2 *buf1, const float2 *__restrict__ tw) {
    return fft_passes<N, 1, INV, T, COMP>(buf0, buf1, tw);
}

// ------------------------------------------------ compact row FFT (one pass body)
// The same Stockham plan, butterflies, twiddle products and rounding as
// fft_row (results agree bit for bit), with the pass stride NS and the
// direction taken at run time: one radix-8 pass body serves every radix-8 pass
// of both transforms, so a kernel with two row FFTs carries two pass bodies
// instead of eight unrolled ones (the unrolled form's code overflows the
// instruction cache in the fused row kernels).  sg = +1 forward, -1 inverse;
// multiplying by sg is exact, and every sum and rounding is that of the
// compile-time form (e.g. the inverse's x - y is formed as x + (-y)).

// v *= exp(-+ i pi / 2) for sg = +1 / -1
__device__ __forceinline__ float2 c_quarter_s(float2 a, float sg) { return make_float2(sg * a.y, -sg * a.x); }

__device__ __forceinline__ void dft4_s(float2 *v, float sg) {
    float2 y0 = c_add(v[0], v[2]), y1 = c_sub(v[0], v[2]);
    float2 y2 = c_add(v[1], v[3]), y3 = c_quarter_s(c_sub(v[1], v[3]), sg);
    v[0] = c_add(y0, y2);
    v[2] = c_sub(y0, y2);
    v[1] = c_add(y1, y3);
    v[3] = c_sub(y1, y3);
}

__device__ __forceinline__ void dft8_s(float2 *v, float sg) {
    float2 a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        a[r] = c_add(v[r], v[r + 4]);
        b[r] = c_sub(v[r], v[r + 4]);
    }
    // b_r *= w8^r, w8 = exp(-+ i pi / 4) (dft8's expressions with y -> sg y)
    {
        const float y = sg * b[1].y;
        b[1] = make_float2(mul_rsqrt2(b[1].x + y), sg * mul_rsqrt2(y - b[1].x));
    }
    b[2] = c_quarter_s(b[2], sg);
    {
        const float y = sg * b[3].y;
        b[3] = make_float2(mul_rsqrt2(y - b[3].x), -sg * mul_rsqrt2(b[3].x + y));
    }
    dft4_s(a, sg);
    dft4_s(b, sg);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        v[2 * m] = a[m];
        v[2 * m + 1] = b[m];
    }
}

template <int R>
__device__ __forceinline__ void dft_small_s(float2 *v, float sg) {
    if (R == 2) {
        dft2<false>(v);
    } else if (R == 4) {
        dft4_s(v, sg);
    } else {
        dft8_s(v, sg);
    }
}

// One radix-R pass over an N-point row at run-time stride NS (> 1: twiddles
// from the pass's table block at tw_pass; tw_rem = the remainders' offset).
template <int R, int N, int T>
__device__ __forceinline__ void stockham_pass_s(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                                const float2 *__restrict__ tw_pass, int tw_rem, int NS, float sg) {
    constexpr int nb = N / R;
#pragma unroll
    for (int jj = 0; jj < (nb + T - 1) / T; ++jj) {
        const int j = (int)threadIdx.x + jj * T;
        if (nb % T == 0 || j < nb) {
            const int k = j & (NS - 1);
            float2 v[R];
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = src[pidx(j + r * nb)];
            if (NS > 1) {
                const float4 *w4 = reinterpret_cast<const float4 *>(tw_pass) + k;
                float2 w[fft_tw_row(R)];
#pragma unroll
                for (int q = 0; q < fft_tw_row(R) / 2; ++q) {
                    const float4 p = __ldg(&w4[q * NS]);
                    w[2 * q] = make_float2(p.x, p.y);
                    w[2 * q + 1] = make_float2(p.z, p.w);
                }
#if NLSE_COMP_TWIDDLE
                const float4 *l4 = w4 + tw_rem / 2;
                float2 wl[fft_tw_row(R)];
#pragma unroll
                for (int q = 0; q < fft_tw_row(R) / 2; ++q) {
                    const float4 p = __ldg(&l4[q * NS]);
                    wl[2 * q] = make_float2(p.x, p.y);
                    wl[2 * q + 1] = make_float2(p.z, p.w);
                }
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    const float2 x = make_float2(w[r - 1].x, sg * w[r - 1].y);
                    const float2 xl = make_float2(wl[r - 1].x, sg * wl[r - 1].y);
#if NLSE_COMP_TWIDDLE == 2
                    v[r] = c_mul_exact(v[r], x, xl);
#else
                    v[r] = c_mul_comp(v[r], x, xl);
#endif
                }
#else
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = c_mul(v[r], make_float2(w[r - 1].x, sg * w[r - 1].y));
#endif
            }
            dft_small_s<R>(v, sg);
            const int d0 = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) dst[pidx(d0 + r * NS)] = v[r];
        }
    }
}

// Full FFT of one row (as fft_row: buf0 in, buf1 scratch, returns the buffer
// holding the unnormalised result); inv selects the direction at run time.
template <int N, int T = NLSE_ROW_THREADS>
__device__ __forceinline__ float2 *fft_row_s(float2 *buf0, float2 *buf1, const float2 *__restrict__ tw, bool inv) {
    const float sg = inv ? -1.0f : 1.0f;
    float2 *src = buf0, *dst = buf1;
    int NS = 1, off = 0;
#pragma unroll 1
    while (fft_radix(N, NS) == 8 && NS < N) {
        stockham_pass_s<8, N, T>(src, dst, tw + off, fft_tw_size(N), NS, sg);
        if (NS > 1) off += NS * fft_tw_row(8);
        NS *= 8;
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    if (NS < N) {
        // the one remaining pass (radix N / NS, 4 or 2)
        if (N / NS == 4) {
            stockham_pass_s<4, N, T>(src, dst, tw + off, fft_tw_size(N), NS, sg);
        } else {
            stockham_pass_s<2, N, T>(src, dst, tw + off, fft_tw_size(N), NS, sg);
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// ------------------------------------------------ register-resident row FFT
// The same Stockham plan, butterflies and twiddle products as fft_row (the
// results agree bit for bit) with the row held in registers: each of the T
// threads keeps P = N / T points, v[m] = point threadIdx.x + T m, on entry and
// on exit.  Butterfly j = threadIdx.x + T q of a pass takes its inputs
// j + r N / R: in the first pass they are the thread's own v[q + r P / R], and
// the last pass's outputs j + r N / R land in v[q + r P / R] again, so the row
// crosses shared memory only between passes (padded buffers A, B, A, ...; one
// barrier each).  Every radix of the plan must divide P.
template <int N, int T>
__host__ __device__ constexpr bool fft_regs_ok() {
    if (N % T != 0 || N / T < 2) return false;
    int passes = 0;
    for (int s = 1; s < N; s *= fft_radix(N, s)) {
        if ((N / T) % fft_radix(N, s) != 0) return false;
        ++passes;
    }
    return passes >= 3;  // at least two exchanges (see fft_regs)
}

template <int N, int NS, bool INV, int T, bool COMP = true>
__device__ __forceinline__ float2 *fft_regs_pass(float2 (&v)[N / T], float2 *src, float2 *dst,
                                                 const float2 *__restrict__ tw) {
    constexpr int P = N / T, R = fft_radix(N, NS), Q = P / R, nb = N / R;
    constexpr bool first = NS == 1, last = NS * R == N;
    static_assert(P % R == 0, "every radix must divide the points per thread");
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = (int)threadIdx.x + q * T;
        const int k = j & (NS - 1);
        float2 y[R];
        if constexpr (first) {
#pragma unroll
            for (int r = 0; r < R; ++r) y[r] = v[q + r * Q];
        } else if constexpr (pass_src_linear(nb)) {
            const float2 *s = src + pidx(j);
#pragma unroll
            for (int r = 0; r < R; ++r) y[r] = s[r * (nb + nb / 16)];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) y[r] = src[pidx(j + r * nb)];
        }
        if (NS > 1) apply_twiddles<R, INV, N, NS, COMP>(y, k, tw);
        dft_small<R, INV>(y);
        if constexpr (last) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[q + r * Q] = y[r];
        } else if constexpr (pass_dst_linear(NS, R)) {
            float2 *d = dst + pidx((j - k) * R + k);
#pragma unroll
            for (int r = 0; r < R; ++r) d[pass_dst_step(NS, r)] = y[r];
        } else {
            const int d0 = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) dst[pidx(d0 + r * NS)] = y[r];
        }
    }
    if constexpr (!last) {
        __syncthreads();
        return fft_regs_pass<N, NS * R, INV, T, COMP>(v, dst, src, tw);
    } else {
        return dst;
    }
}

// Unnormalised FFT of the row in v (layout above).  The first pass writes A
// without a barrier, so no thread may still read A.  Returns a buffer that was
// last read before the final barrier: free to write at once (the other one
// only after a barrier).
template <int N, bool INV, int T = NLSE_ROW_THREADS, bool COMP = true>
__device__ __forceinline__ float2 *fft_regs(float2 (&v)[N / T], float2 *A, float2 *B,
                                            const float2 *__restrict__ tw) {
    static_assert(fft_regs_ok<N, T>(), "row length not supported by the register FFT");
    return fft_regs_pass<N, 1, INV, T, COMP>(v, B, A, tw);
}

// Entry e (a float2 index) of the twiddle table of an N-point row (host or
// device, FP64 then rounded): the pass, row k and r it stands for give
// m = r k N / (NS R) (layout above: float4 q of row k at q NS + k).
__host__ __device__ inline void fft_tw_entry(int N, int e, int *m_out) {
    int off = 0, m = -1;
    for (int NS = 1; NS < N; NS *= fft_radix(N, NS)) {
        if (NS == 1) continue;
        const int R = fft_radix(N, NS), row = fft_tw_row(R), n = NS * row;
        if (e < off + n) {
            const int el = e - off, f = el >> 1, q = f / NS, k = f % NS, r = 2 * q + (el & 1) + 1;
            m = r < R ? r * k * (N / (NS * R)) : -1;  // -1: padding
            break;
        }
        off += n;
    }
    *m_out = m;
}

// Dispatch a runtime power-of-two size to a kernel template instantiated for
// N = 16 .. 8192 (the macro body sees the compile-time constant NT).
#define NLSE_DISPATCH_NT(logn, ...)                          \
    switch (logn) {                                          \
        case 4: { constexpr int NT = 16; __VA_ARGS__; break; }    \
        case 5: { constexpr int NT = 32; __VA_ARGS__; break; }    \
        case 6: { constexpr int NT = 64; __VA_ARGS__; break; }    \
        case 7: { constexpr int NT = 128; __VA_ARGS__; break; }   \
        case 8: { constexpr int NT = 256; __VA_ARGS__; break; }   \
        case 9: { constexpr int NT = 512; __VA_ARGS__; break; }   \
        case 10: { constexpr int NT = 1024; __VA_ARGS__; break; } \
        case 11: { constexpr int NT = 2048; __VA_ARGS__; break; } \
        case 12: { constexpr int NT = 4096; __VA_ARGS__; break; } \
        case 13: { constexpr int NT = 8192; __VA_ARGS__; break; } \
        default: return cudaErrorInvalidValue;               \
    }

// The same for the full-physics kernels (N_t <= 4096: three row buffers and
// the per-thread register arrays of the RK stages).
#define NLSE_DISPATCH_NT_FULL(logn, ...)                          \
    switch (logn) {                                               \
        case 4: { constexpr int NT = 16; __VA_ARGS__; break; }    \
        case 5: { constexpr int NT = 32; __VA_ARGS__; break; }    \
        case 6: { constexpr int NT = 64; __VA_ARGS__; break; }    \
        case 7: { constexpr int NT = 128; __VA_ARGS__; break; }   \
        case 8: { constexpr int NT = 256; __VA_ARGS__; break; }   \
        case 9: { constexpr int NT = 512; __VA_ARGS__; break; }   \
        case 10: { constexpr int NT = 1024; __VA_ARGS__; break; } \
        case 11: { constexpr int NT = 2048; __VA_ARGS__; break; } \
        case 12: { constexpr int NT = 4096; __VA_ARGS__; break; } \
        default: return cudaErrorInvalidValue;                    \
    }
