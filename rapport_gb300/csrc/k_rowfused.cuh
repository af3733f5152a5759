// Fused row kernels of the split-BF16 path (one CTA per radius r).
//
// Between z-steps the field is kept in the Omega domain, w = F[u], stored
// planar (row r = Re, row Nr + r = Im) in FP32 plus its BF16 hi/lo terms --
// the B operand of the tensor-core product E' w'.  One z-step of
// Integrator.propagate (update_plasma + step, integrator.py:138-158) becomes
//
//   G1      D  = E' w                                (k_gemm_tc)
//   row_nl  x  = P_t (w + D); u = F^-1[x]; u <- NL(u, rho); y = F[u]
//   G2      D  = E' y                                (k_gemm_tc)
//   row_nx  w' = mask_r P_t (y + D); u' = F^-1[w']; rho <- march(|u'|^2)
//
// where P_t = e^{i dk dz/2} spec_mask, the identity part of M = I + E is
// added here exactly in FP32, and row_nx's march is the NEXT iteration's
// update_plasma (the entry kernel does the first one).  Each row kernel reads
// and writes its row once (HBM) and does the FFTs, the nonlinear block and the
// scan in shared memory.
//
// Templates only: each N_t is instantiated in a translation unit of its own
// (k_row_n*.cu, RowKernels<NT>), so the sizes compile in parallel; the
// runtime dispatch over N_t is in k_rowfused.cu.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fullnl_impl.cuh"
#include "scan_impl.cuh"


// Exponent sb of the FP16 field terms of GEMM input g (split-FP16 form): the
// largest |w| of input g - 1 (one z half-step earlier) maps to below 2^7, so
// the terms stay below FP16's 65504 unless |w| grows 512-fold in a half step
// (an overflow is counted in scale[NLSE_SC_OVF]); values down to 2^-17 of the
// maximum keep all 22 bits of the two terms.
__device__ __forceinline__ int f16_field_exp(const int *scale, int g) {
    const float prev = __int_as_float(__ldcg(&scale[NLSE_SC_MAX + (g + 2) % 3]));
    if (!(prev > 0.0f) || !isfinite(prev)) return 0;
    int e;
    frexpf(prev, &e);  // prev < 2^e
    return min(max(7 - e, -100), 100);
}

// Threads per CTA of row_entry / row_next: 8 points each from N_t = 2048 on
// (256, 512 at 4096, 1024 at 8192), so rows whose buffers admit only 1-2 CTAs
// per SM still give it 32 warps; 256 below 2048.  The full-physics row
// kernels (N_t <= 4096) keep 256.
template <int NT>
__host__ __device__ constexpr int row_threads() {
    return NT >= 8192 ? 1024 : (NT == 4096 ? 512 : NLSE_ROW_THREADS);
}

// row_nl (no march, two shared-memory row buffers) measured faster with 256
// threads up to N_t = 4096 (three CTAs per SM there), 1024 at 8192.
template <int NT>
__host__ __device__ constexpr int row_threads_nl() {
    return NT >= 8192 ? 1024 : NLSE_ROW_THREADS;
}

// Block-wide max of a non-negative float (all threads, up to 1024; result valid in thread 0).
__device__ __forceinline__ float block_max(float v) {
    __shared__ float red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = fmaxf(v, red[w]);
    return v;
}

// Factor that removes the product's scaling: 1 in the split-BF16 form, else
// 2^-(sa + sb_g) (merged operator: field exponent of input g) or 2^-(sa + sv_g)
// (space-time focusing: exponent of the second product's input).  Either way
// the product is E w and the row kernel adds the identity part w exactly.
__device__ __forceinline__ float product_scale(const RowFusedArgs &a, int g_in) {
    if (!a.f16) return 1.0f;
    const int e = __ldcg(&a.scale[(a.stf ? NLSE_SC_VB : NLSE_SC_SB) + g_in % 2]);
    return ldexpf(1.0f, -(__ldcg(&a.scale[NLSE_SC_SA]) + e));
}

// FP32 planar rows + the 16-bit hi/lo terms (the GEMM's B operand) of one
// complex row held in smem (padded indexing); two points per thread per
// iteration.  BF16 form: hi = bf16(w), lo = bf16(w - hi).  Split-FP16 form:
// the same of w 2^sb in FP16, with the row's max |w| and the bookkeeping of
// the scale cells (g_out = the index of this GEMM input).
template <int NT>
__device__ __forceinline__ void store_state_row(const float2 *s, int r, const RowFusedArgs &a, float *F32,
                                                __nv_bfloat16 *Fb, int g_out) {
    const size_t rows = 2 * (size_t)a.Nrp;
    float *re = F32 + (size_t)r * NT, *im = F32 + ((size_t)a.Nrp + r) * NT;
    __nv_bfloat16 *hre = Fb + (size_t)r * NT, *him = Fb + ((size_t)a.Nrp + r) * NT;
    __nv_bfloat16 *lre = hre + rows * NT, *lim = him + rows * NT;
    if (!a.f16) {
        for (int t = 2 * threadIdx.x; t < NT; t += 2 * blockDim.x) {
            const float2 v0 = s[pidx(t)], v1 = s[pidx(t + 1)];
            *reinterpret_cast<float2 *>(re + t) = make_float2(v0.x, v1.x);
            *reinterpret_cast<float2 *>(im + t) = make_float2(v0.y, v1.y);
            const __nv_bfloat162 hx = __floats2bfloat162_rn(v0.x, v1.x), hy = __floats2bfloat162_rn(v0.y, v1.y);
            *reinterpret_cast<__nv_bfloat162 *>(hre + t) = hx;
            *reinterpret_cast<__nv_bfloat162 *>(him + t) = hy;
            *reinterpret_cast<__nv_bfloat162 *>(lre + t) =
                __floats2bfloat162_rn(v0.x - __low2float(hx), v1.x - __high2float(hx));
            *reinterpret_cast<__nv_bfloat162 *>(lim + t) =
                __floats2bfloat162_rn(v0.y - __low2float(hy), v1.y - __high2float(hy));
        }
        return;
    }
    const int sb = f16_field_exp(a.scale, g_out);
    const float sc = ldexpf(1.0f, sb);
    float mx = 0.0f;
    for (int t = 2 * threadIdx.x; t < NT; t += 2 * blockDim.x) {
        const float2 v0 = s[pidx(t)], v1 = s[pidx(t + 1)];
        *reinterpret_cast<float2 *>(re + t) = make_float2(v0.x, v1.x);
        *reinterpret_cast<float2 *>(im + t) = make_float2(v0.y, v1.y);
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
    mx = block_max(mx);
    if (threadIdx.x == 0) {
        atomicMax(&a.scale[NLSE_SC_MAX + g_out % 3], __float_as_int(mx));
        if (ovf) atomicAdd(&a.scale[NLSE_SC_OVF], 1);
        if (r == 0) {
            a.scale[NLSE_SC_SB + g_out % 2] = sb;
            a.scale[NLSE_SC_MAX + (g_out + 1) % 3] = 0;  // the slot input g_out + 1 will fill
        }
    }
}

// s[t] = scale * P_t[t] * ((F32 + D) row r as complex), padded indexing.  In
// the split-FP16 form D carries 2^(sa + sb) of input g_in, removed here.
template <int NT>
__device__ __forceinline__ void load_mw_row(float2 *s, int r, const RowFusedArgs &a, const float *F32,
                                            const float *D, float scale, int g_in) {
    const float ds = product_scale(a, g_in);
    const float *fr = F32 + (size_t)r * NT, *fi = F32 + ((size_t)a.Nrp + r) * NT;
    const float *dr = D + (size_t)r * NT, *di = D + ((size_t)a.Nrp + r) * NT;
    for (int t = 2 * threadIdx.x; t < NT; t += 2 * blockDim.x) {
        const float2 xr = *reinterpret_cast<const float2 *>(fr + t), xi = *reinterpret_cast<const float2 *>(fi + t);
        const float2 yr = *reinterpret_cast<const float2 *>(dr + t), yi = *reinterpret_cast<const float2 *>(di + t);
        const float4 pt = __ldg(reinterpret_cast<const float4 *>(a.Pt + t));
#if NLSE_COMP_TWIDDLE
        const float4 pl = __ldg(reinterpret_cast<const float4 *>(a.Pt + NT + t));
        s[pidx(t)] = c_scale(c_mul_comp(make_float2(fmaf(yr.x, ds, xr.x), fmaf(yi.x, ds, xi.x)),
                                        make_float2(pt.x, pt.y), make_float2(pl.x, pl.y)),
                             scale);
        s[pidx(t + 1)] = c_scale(c_mul_comp(make_float2(fmaf(yr.y, ds, xr.y), fmaf(yi.y, ds, xi.y)),
                                            make_float2(pt.z, pt.w), make_float2(pl.z, pl.w)),
                                 scale);
#else
        s[pidx(t)] = c_scale(c_mul(make_float2(fmaf(yr.x, ds, xr.x), fmaf(yi.x, ds, xi.x)), make_float2(pt.x, pt.y)),
                             scale);
        s[pidx(t + 1)] =
            c_scale(c_mul(make_float2(fmaf(yr.y, ds, xr.y), fmaf(yi.y, ds, xi.y)), make_float2(pt.z, pt.w)), scale);
#endif
    }
}

// Carrier march of the intensities already written to sI (scan layout): scan
// in the scratch Rb (a complex row buffer no thread reads any more); writes
// rho row r.
template <int NT>
__device__ __forceinline__ void march_scan(float *sI, float2 *Rb, int r, const RowFusedArgs &a, float *rho) {
    constexpr int S = scan_span(NT, row_threads<NT>());
    using Sh = ScanShape<NT, row_threads<NT>()>;
    float *sW = sI + S;
    __syncthreads();
    float *sx = reinterpret_cast<float *>(Rb);
    scan_row_ct<NT, row_threads<NT>()>(sI, sW, sx, a.sc, a.lut, 0.0f, a.stats);
    float *gr = rho + (size_t)r * NT;
    for (int t = threadIdx.x; t < NT; t += row_threads<NT>()) gr[t] = sx[Sh::slot(t)];
}

// Carrier march of the physical row held (unnormalised by inv) in R; scratch
// in the other FFT buffer O; writes rho row r.
template <int NT>
__device__ __forceinline__ void march_row(float2 *R, float2 *O, float inv, int r, const RowFusedArgs &a,
                                          float *rho) {
    using Sh = ScanShape<NT, row_threads<NT>()>;
    float *sI = reinterpret_cast<float *>(O);
    for (int t = threadIdx.x; t < NT; t += row_threads<NT>()) {
        const float2 v = c_scale(R[pidx(t)], inv);
        sI[Sh::slot(t)] = fmaf(v.x, v.x, v.y * v.y) * a.sc.invE2;
    }
    march_scan<NT>(sI, R, r, a, rho);
}

// 2 padded complex row buffers.  The march aliases its arrays into them (the
// intensities and rates into one, the densities into the other): 2 * span
// floats must fit in fft_slots(NT) float2, which holds for every NT >= 16 with
// 256 threads.  (The sweep's affine maps stay in registers, scan_row_ct.)
template <int NT>
__host__ __device__ constexpr size_t row_smem_bytes(bool with_march) {
    constexpr int span = scan_span(NT, row_threads<NT>());
    static_assert(2 * span <= 2 * fft_slots(NT), "scan arrays must fit in the FFT buffers");
    (void)with_march;
    return 2 * (size_t)fft_slots(NT) * sizeof(float2);
}

// ------------------------------------------------ register-resident row_next
// From N_t = 2048 on (8 points per thread) row_next keeps its row in registers:
// thread tid of T holds the points tid + T m.  Loads, the state stores, the
// inverse FFT (fft_regs), the physical field and the march's intensities act
// on those points in place, so the row crosses shared memory only inside the
// FFT; the arithmetic per point is that of the shared-memory body (results
// agree bit for bit), ~10 % faster at 1024 x 2048.  (For row_nl the
// shared-memory body with its two-point vector accesses measured faster.)
template <int NT>
__host__ __device__ constexpr bool row_regs() {
    return fft_regs_ok<NT, row_threads<NT>()>() && NT / row_threads<NT>() == 8;
}

template <int NT, int T>
__device__ __forceinline__ void load_mw_regs(float2 (&v)[NT / T], int r, const RowFusedArgs &a,
                                             const float *F32, const float *D, float scale, int g_in) {
    const float ds = product_scale(a, g_in);
    const float *fr = F32 + (size_t)r * NT, *fi = F32 + ((size_t)a.Nrp + r) * NT;
    const float *dr = D + (size_t)r * NT, *di = D + ((size_t)a.Nrp + r) * NT;
#pragma unroll
    for (int m = 0; m < NT / T; ++m) {
        const int t = (int)threadIdx.x + m * T;
        const float2 x = make_float2(fmaf(dr[t], ds, fr[t]), fmaf(di[t], ds, fi[t]));
        const float2 pt = __ldg(a.Pt + t);
#if NLSE_COMP_TWIDDLE
        v[m] = c_scale(c_mul_comp(x, pt, __ldg(a.Pt + NT + t)), scale);
#else
        v[m] = c_scale(c_mul(x, pt), scale);
#endif
    }
}

template <int NT, int T>
__device__ __forceinline__ void store_state_regs(const float2 (&v)[NT / T], int r,
                                                 const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, int g_out) {
    const size_t rows = 2 * (size_t)a.Nrp;
    float *re = F32 + (size_t)r * NT, *im = F32 + ((size_t)a.Nrp + r) * NT;
    __nv_bfloat16 *hre = Fb + (size_t)r * NT, *him = Fb + ((size_t)a.Nrp + r) * NT;
    __nv_bfloat16 *lre = hre + rows * NT, *lim = him + rows * NT;
    if (!a.f16) {
#pragma unroll
        for (int m = 0; m < NT / T; ++m) {
            const int t = (int)threadIdx.x + m * T;
            re[t] = v[m].x;
            im[t] = v[m].y;
            const __nv_bfloat16 hx = __float2bfloat16_rn(v[m].x), hy = __float2bfloat16_rn(v[m].y);
            hre[t] = hx;
            him[t] = hy;
            lre[t] = __float2bfloat16_rn(v[m].x - __bfloat162float(hx));
            lim[t] = __float2bfloat16_rn(v[m].y - __bfloat162float(hy));
        }
        return;
    }
    __half *fre = reinterpret_cast<__half *>(hre), *fim = reinterpret_cast<__half *>(him);
    __half *gre = reinterpret_cast<__half *>(lre), *gim = reinterpret_cast<__half *>(lim);
    const int sb = f16_field_exp(a.scale, g_out);
    const float sc = ldexpf(1.0f, sb);
    float mx = 0.0f;
#pragma unroll
    for (int m = 0; m < NT / T; ++m) {
        const int t = (int)threadIdx.x + m * T;
        re[t] = v[m].x;
        im[t] = v[m].y;
        mx = fmaxf(mx, fmaxf(fabsf(v[m].x), fabsf(v[m].y)));
        const float x = v[m].x * sc, y = v[m].y * sc;
        const __half hx = __float2half_rn(x), hy = __float2half_rn(y);
        fre[t] = hx;
        fim[t] = hy;
        gre[t] = __float2half_rn(x - __half2float(hx));
        gim[t] = __float2half_rn(y - __half2float(hy));
    }
    // a finite value above 65504 after scaling overflowed its FP16 term
    const int ovf = __syncthreads_or(isfinite(mx) && !(mx * sc <= 65504.0f));
    mx = block_max(mx);
    if (threadIdx.x == 0) {
        atomicMax(&a.scale[NLSE_SC_MAX + g_out % 3], __float_as_int(mx));
        if (ovf) atomicAdd(&a.scale[NLSE_SC_OVF], 1);
        if (r == 0) {
            a.scale[NLSE_SC_SB + g_out % 2] = sb;
            a.scale[NLSE_SC_MAX + (g_out + 1) % 3] = 0;  // the slot input g_out + 1 will fill
        }
    }
}

template <int NT>
__device__ __forceinline__ void row_next_regs(const RowFusedArgs &a, int r, float *__restrict__ F32,
                                              __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
                                              float *__restrict__ rho, float2 *__restrict__ u_out, int write_state,
                                              int do_scan, int apply_mask, int g) {
    constexpr int T = row_threads<NT>();
    extern __shared__ float2 sm2[];
    float2 *A = sm2, *B = sm2 + fft_slots(NT);
    float2 v[NT / T];
    load_mw_regs<NT, T>(v, r, a, F32, D, apply_mask ? __ldg(&a.mask_r[r]) : 1.0f, g);
    if (write_state) store_state_regs<NT, T>(v, r, a, F32, Fb, g + 1);
    if (!do_scan && !u_out) return;
    // a physical field that only feeds the march (rebuilt from it every z-step)
    // takes plain twiddle products (see apply_twiddles); one handed to the
    // caller (the state of the next call) the compensated ones
    float2 *F = u_out ? fft_regs<NT, true, row_threads<NT>(), true>(v, A, B, a.tw)
                      : fft_regs<NT, true, row_threads<NT>(), false>(v, A, B, a.tw);
    const float inv = 1.0f / (float)NT;
    if (u_out) {
        float2 *gu = u_out + (size_t)r * NT;
#pragma unroll
        for (int m = 0; m < NT / row_threads<NT>(); ++m) gu[threadIdx.x + m * row_threads<NT>()] = c_scale(v[m], inv);
    }
    if (!do_scan) return;
    using Sh = ScanShape<NT, row_threads<NT>()>;
    float *sI = reinterpret_cast<float *>(F);
#pragma unroll
    for (int m = 0; m < NT / row_threads<NT>(); ++m) {
        const float2 w = c_scale(v[m], inv);
        sI[Sh::slot((int)threadIdx.x + m * row_threads<NT>())] = fmaf(w.x, w.x, w.y * w.y) * a.sc.invE2;
    }
    march_scan<NT>(sI, F == A ? B : A, r, a, rho);
}

// CTAs per SM the row kernels are compiled for: 6 (40 registers at 256
// threads: more warps to hide the latency of the row's loads and barriers),
// fewer when the shared memory admits fewer (228 KB per SM, 1 KB reserved per
// CTA), and for 512 / 1024 threads no more than leave 64 registers a thread.
template <int NT>
__host__ __device__ constexpr int row_min_blocks(bool with_march) {
    const int T = with_march ? row_threads<NT>() : row_threads_nl<NT>();
    const int by_smem = (228 * 1024) / (int)(row_smem_bytes<NT>(with_march) + 1024);
    const int cap = T >= 512 ? 65536 / (T * 64) : 6;
    return by_smem < cap ? by_smem : cap;
}

// ------------------------------------------------ row plans (autotuned per N_t)
// Each of row_nl / row_next has two or three plans of the same transforms and
// point arithmetic (results agree bit for bit; the choice is pure speed):
//   row_nl   plan 0: shared-memory body, row_threads_nl threads (two points per
//                    thread per access), compile-time FFT passes;
//            plan 1: register-resident body, N_t / 8 threads (from N_t = 512);
//            plan 2: plan 0 with the compact FFT (one run-time pass body for
//                    both transforms: a fraction of the instruction footprint).
//   row_next plan 0: register-resident from N_t = 2048, else shared memory;
//            plan 1: the shared-memory body at the same thread count (N_t >= 2048).
// The thread count of row_next (its carrier march is chunked per thread) is
// the same in both plans.
template <int NT>
__host__ __device__ constexpr bool nl_plan1_ok() {
    return NT >= 512 && fft_regs_ok<NT, NT / 8>();
}

template <int NT>
__host__ __device__ constexpr bool next_plan1_ok() {
    return row_regs<NT>();
}

template <int NT, int PLAN>
__host__ __device__ constexpr bool nl_plan_ok() {
    return PLAN == 0 || PLAN == 2 || (PLAN == 1 && nl_plan1_ok<NT>());
}

template <int NT, int PLAN>
__host__ __device__ constexpr int nl_threads() {
    return (PLAN == 1 && nl_plan1_ok<NT>()) ? NT / 8 : row_threads_nl<NT>();
}

// CTAs per SM a kernel of T threads and the given dynamic shared memory is
// compiled for: what the shared memory and the 2048 threads per SM admit, at
// no fewer than 40 registers a thread (64 from 512 threads on).
template <int T>
__host__ __device__ constexpr int row_min_blocks_t(size_t smem) {
    const int by_smem = (228 * 1024) / (int)(smem + 1024);
    const int by_regs = 65536 / (T * (T >= 512 ? 64 : 40));
    const int by_thr = 2048 / T;
    const int m = by_smem < by_regs ? by_smem : by_regs;
    const int n = m < by_thr ? m : by_thr;
    return n > 1 ? n : 1;
}

template <int NT, int PLAN>
__host__ __device__ constexpr int nl_min_blocks() {
    return PLAN == 1 && nl_plan1_ok<NT>() ? row_min_blocks_t<nl_threads<NT, PLAN>()>(row_smem_bytes<NT>(false))
                                          : row_min_blocks<NT>(false);
}

// Entry: physical u (interleaved) -> w = F[u] (state); optionally rho = march(|u|^2).
template <int NT>
__device__ __forceinline__ void row_entry_body(const RowFusedArgs &a, int r, const float2 *__restrict__ u,
                                               float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb,
                                               float *__restrict__ rho, int do_scan) {
    extern __shared__ float2 sm2[];
    float2 *b0 = sm2, *b1 = sm2 + fft_slots(NT);
    const float2 *g = u + (size_t)r * NT;
    for (int t = 2 * threadIdx.x; t < NT; t += 2 * blockDim.x) {
        const float4 v = *reinterpret_cast<const float4 *>(g + t);
        b0[pidx(t)] = make_float2(v.x, v.y);
        b0[pidx(t + 1)] = make_float2(v.z, v.w);
    }
    __syncthreads();
    float2 *R = fft_row<NT, false, row_threads<NT>()>(b0, b1, a.tw);
    store_state_row<NT>(R, r, a, F32, Fb, 0);
    if (!do_scan) return;
    __syncthreads();
    // the march needs the physical field: reload it into the free buffer
    float2 *O = R == b0 ? b1 : b0;
    for (int t = threadIdx.x; t < NT; t += blockDim.x) O[pidx(t)] = g[t];
    __syncthreads();
    march_row<NT>(O, R, 1.0f, r, a, rho);
}

// row_nl plan 1: the row held in registers, 8 points per thread (N_t / 8
// threads): the inverse FFT ends and the forward FFT starts in registers, so
// the nonlinear block acts on the thread's own points and the row crosses
// shared memory only between FFT passes.
template <int NT>
__device__ __forceinline__ void row_nl_regs_body(const RowFusedArgs &a, int r, float *__restrict__ F32,
                                                 __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
                                                 const float *__restrict__ rho, const float *__restrict__ rho_s,
                                                 int g) {
    constexpr int T = NT / 8, P = 8;
    extern __shared__ float2 sm2[];
    float2 *A = sm2, *B = sm2 + fft_slots(NT);
    float2 v[P];
    load_mw_regs<NT, T>(v, r, a, F32, D, 1.0f / (float)NT, g);
    float2 *F = fft_regs<NT, true, T>(v, A, B, a.tw);
    const float *gr = rho + (size_t)r * NT;
    const float *gs = rho_s ? rho_s + (size_t)r * NT : nullptr;
    // The nonlinear block runs rolled (its unrolled copies overflow the
    // instruction cache), which would index v at run time and move it to
    // local memory: the thread's points go through their own slots of F
    // instead (F was last read before the inverse transform's final barrier,
    // and each thread reads back only what it wrote).
#pragma unroll
    for (int m = 0; m < P; ++m) F[pidx((int)threadIdx.x + m * T)] = v[m];
#pragma unroll 1
    for (int m = 0; m < P; ++m) {
        const int t = (int)threadIdx.x + m * T;
        F[pidx(t)] = nl_point(F[pidx(t)], gr[t], gs ? gs[t] : 0.0f, a.dz, a.nl, a.pchip);
    }
#pragma unroll
    for (int m = 0; m < P; ++m) v[m] = F[pidx((int)threadIdx.x + m * T)];
    // the forward transform's first pass writes F without a barrier: every
    // thread must have read its points back first
    __syncthreads();
    fft_regs<NT, false, T>(v, F, F == A ? B : A, a.tw);
    store_state_regs<NT, T>(v, r, a, F32, Fb, g + 1);
}

// First half step's spectral end + the nonlinear block + forward FFT.
template <int NT, int PLAN = 0>
__device__ __forceinline__ void row_nl_body(const RowFusedArgs &a, int r, float *__restrict__ F32,
                                            __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
                                            const float *__restrict__ rho, const float *__restrict__ rho_s, int g) {
    if constexpr (PLAN == 1 && nl_plan1_ok<NT>()) {
        row_nl_regs_body<NT>(a, r, F32, Fb, D, rho, rho_s, g);
        return;
    }
    extern __shared__ float2 sm2[];
    float2 *b0 = sm2, *b1 = sm2 + fft_slots(NT);
    load_mw_row<NT>(b0, r, a, F32, D, 1.0f / (float)NT, g);
    __syncthreads();
    float2 *R = PLAN == 2 ? fft_row_s<NT, row_threads_nl<NT>()>(b0, b1, a.tw, true)
                          : fft_row<NT, true, row_threads_nl<NT>()>(b0, b1, a.tw);
    const float *gr = rho + (size_t)r * NT;
    const float *gs = rho_s ? rho_s + (size_t)r * NT : nullptr;
    // kept rolled: the RK4 block is long, and unrolled copies of it (with the
    // two transforms around it) overflow the instruction cache
#pragma unroll 1
    for (int t = 2 * threadIdx.x; t < NT; t += 2 * blockDim.x) {
        const float2 rr = *reinterpret_cast<const float2 *>(gr + t);
        const float2 rs = gs ? *reinterpret_cast<const float2 *>(gs + t) : make_float2(0.0f, 0.0f);
        R[pidx(t)] = nl_point(R[pidx(t)], rr.x, rs.x, a.dz, a.nl, a.pchip);
        R[pidx(t + 1)] = nl_point(R[pidx(t + 1)], rr.y, rs.y, a.dz, a.nl, a.pchip);
    }
    __syncthreads();
    float2 *Y = PLAN == 2 ? fft_row_s<NT, row_threads_nl<NT>()>(R, R == b0 ? b1 : b0, a.tw, false)
                          : fft_row<NT, false, row_threads_nl<NT>()>(R, R == b0 ? b1 : b0, a.tw);
    store_state_row<NT>(Y, r, a, F32, Fb, g + 1);
}

// Second half step's spectral end + mask_r: the next state w', and optionally
// the physical field (u_out) and the next carrier march (rho).
template <int NT, int PLAN = 0>
__device__ __forceinline__ void row_next_body(const RowFusedArgs &a, int r, float *__restrict__ F32,
                                              __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
                                              float *__restrict__ rho, float2 *__restrict__ u_out, int write_state,
                                              int do_scan, int apply_mask, int g) {
    if constexpr (PLAN == 0 && row_regs<NT>()) {
        row_next_regs<NT>(a, r, F32, Fb, D, rho, u_out, write_state, do_scan, apply_mask, g);
        return;
    }
    extern __shared__ float2 sm2[];
    float2 *b0 = sm2, *b1 = sm2 + fft_slots(NT);
    load_mw_row<NT>(b0, r, a, F32, D, apply_mask ? __ldg(&a.mask_r[r]) : 1.0f, g);
    __syncthreads();
    if (write_state) store_state_row<NT>(b0, r, a, F32, Fb, g + 1);
    if (!do_scan && !u_out) return;
    // plain twiddle products when the physical field only feeds the march (as in row_next_regs)
    float2 *R = u_out ? fft_row<NT, true, row_threads<NT>(), true>(b0, b1, a.tw)
                      : fft_row<NT, true, row_threads<NT>(), false>(b0, b1, a.tw);
    const float inv = 1.0f / (float)NT;
    if (u_out) {
        float2 *g = u_out + (size_t)r * NT;
        for (int t = 2 * threadIdx.x; t < NT; t += 2 * blockDim.x) {
            const float2 v0 = c_scale(R[pidx(t)], inv), v1 = c_scale(R[pidx(t + 1)], inv);
            *reinterpret_cast<float4 *>(g + t) = make_float4(v0.x, v0.y, v1.x, v1.y);
        }
    }
    if (!do_scan) return;
    march_row<NT>(R, R == b0 ? b1 : b0, inv, r, a, rho);
}

// row_nl with the full-physics nonlinear block (Raman / self-steepening in
// split(); three row buffers).
template <int NT>
__device__ __forceinline__ void row_nl_full_body(const RowFusedArgs &a, int r, float *__restrict__ F32,
                                                 __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
                                                 const float *__restrict__ rho, const float *__restrict__ rho_s,
                                                 int g) {
    extern __shared__ float2 sm2[];
    // the block's constants, read at every point of every RK stage by the
    // out-of-line right-hand side: a copy in shared memory (a reference into
    // the kernel's parameters would reload them from there at each use)
    __shared__ NLParams s_nl;
    __shared__ FullTabs s_ft;
    if (threadIdx.x == 0) {
        s_nl = a.nl;
        s_ft = a.ft;
    }
    const FullRows m = full_rows<NT>(sm2);
    load_mw_row<NT>(m.B0, r, a, F32, D, 1.0f / (float)NT, g);
    __syncthreads();
    const float2 *R = fft_row<NT, true, full_threads<NT>()>(m.B0, m.B1, a.tw);
    for (int t = threadIdx.x; t < NT; t += full_threads<NT>()) m.U[t] = R[pidx(t)];
    __syncthreads();
    nl_block_full<NT>(m, rho + (size_t)r * NT, rho_s ? rho_s + (size_t)r * NT : nullptr, a.dz, s_nl, a.pchip,
                      s_ft, a.tw);
    for (int t = threadIdx.x; t < NT; t += full_threads<NT>()) m.B0[pidx(t)] = m.U[t];
    __syncthreads();
    float2 *Y = fft_row<NT, false, full_threads<NT>()>(m.B0, m.B1, a.tw);
    store_state_row<NT>(Y, r, a, F32, Fb, g + 1);
}

template <int NT>
__global__ void __launch_bounds__(full_threads<NT>(), full_min_blocks<NT>())
k_row_nl_full(RowFusedArgs a, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
              const float *__restrict__ rho, int g) {
    row_nl_full_body<NT>(a, blockIdx.x, F32, Fb, D, rho, a.rho_s, g);
}

template <int NT>
__global__ void __launch_bounds__(row_threads<NT>())
k_row_entry(RowFusedArgs a, const float2 *__restrict__ u, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb,
            float *__restrict__ rho, int do_scan) {
    row_entry_body<NT>(a, blockIdx.x, u, F32, Fb, rho, do_scan);
}

template <int NT, int PLAN>
__global__ void __launch_bounds__(nl_threads<NT, PLAN>(), nl_min_blocks<NT, PLAN>())
k_row_nl(RowFusedArgs a, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
         const float *__restrict__ rho, int g) {
    row_nl_body<NT, PLAN>(a, blockIdx.x, F32, Fb, D, rho, a.rho_s, g);
}

template <int NT, int PLAN>
__global__ void __launch_bounds__(row_threads<NT>(), row_min_blocks<NT>(true))
k_row_next(RowFusedArgs a, float *__restrict__ F32, __nv_bfloat16 *__restrict__ Fb, const float *__restrict__ D,
           float *__restrict__ rho, float2 *__restrict__ u_out, int write_state, int do_scan, int apply_mask, int g) {
    row_next_body<NT, PLAN>(a, blockIdx.x, F32, Fb, D, rho, u_out, write_state, do_scan, apply_mask, g);
}

// ------------------------------------------------------------------ batched (many pulses, one time-grid class)
// work[b] = (pulse, row) for CTA b, the pulse an index into the launch's table
// T (its arguments, read through the constant cache) and into C (the caller's
// buffers for this call); every pulse of the class has the same N_t.
template <int NT>
__global__ void __launch_bounds__(row_threads<NT>())
k_row_entry_b(const __grid_constant__ PulseTable T, const BatchCall *__restrict__ C, const int2 *__restrict__ work,
              int do_scan) {
    const int2 w = work[blockIdx.x];
    const BatchPulse &q = T.p[w.x];
    const BatchCall c = C[w.x];
    // exciton channel: its two-population march runs as a kernel of its own
    row_entry_body<NT>(q.a, w.y, c.u, q.F32, q.Fb, c.rho, do_scan && !q.ste_work);
}

template <int NT, int PLAN>
__global__ void __launch_bounds__(nl_threads<NT, PLAN>(), nl_min_blocks<NT, PLAN>())
k_row_nl_b(const __grid_constant__ PulseTable T, const BatchCall *__restrict__ C, const int2 *__restrict__ work,
           int g) {
    const int2 w = work[blockIdx.x];
    const BatchPulse &q = T.p[w.x];
    row_nl_body<NT, PLAN>(q.a, w.y, q.F32, q.Fb, q.D, C[w.x].rho, C[w.x].rho_s, g);
}

template <int NT, int PLAN>
__global__ void __launch_bounds__(row_threads<NT>(), row_min_blocks<NT>(true))
k_row_next_b(const __grid_constant__ PulseTable T, const BatchCall *__restrict__ C, const int2 *__restrict__ work,
             int last, int g) {
    const int2 w = work[blockIdx.x];
    const BatchPulse &q = T.p[w.x];
    const BatchCall c = C[w.x];
    if (q.ste_work)  // exciton channel: hand the physical field to the two-population march
        row_next_body<NT, PLAN>(q.a, w.y, q.F32, q.Fb, q.D, c.rho, last ? c.u : q.ste_work, !last, 0, 1, g);
    else
        row_next_body<NT, PLAN>(q.a, w.y, q.F32, q.Fb, q.D, c.rho, last ? c.u : nullptr, !last, !last, 1, g);
}

// Pulses with the full-physics terms (Raman / self-steepening; one time-grid class).
template <int NT>
__global__ void __launch_bounds__(full_threads<NT>(), full_min_blocks<NT>())
k_row_nl_full_b(const __grid_constant__ PulseTable T, const BatchCall *__restrict__ C,
                const int2 *__restrict__ work, int g) {
    const int2 w = work[blockIdx.x];
    const BatchPulse &q = T.p[w.x];
    row_nl_full_body<NT>(q.a, w.y, q.F32, q.Fb, q.D, C[w.x].rho, C[w.x].rho_s, g);
}

template <typename K>
static cudaError_t set_smem(K *fn, size_t bytes) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    return e;
}

// Host launchers of the row kernels for one compile-time N_t (the arguments
// are those of the launch_row_* dispatchers in nlse_internal.cuh).
template <int NT>
struct RowKernels {
    static cudaError_t entry(const RowFusedArgs &a, const float2 *u, float *F32, __nv_bfloat16 *Fb, float *rho,
                             int do_scan, cudaStream_t st);
    static cudaError_t nl(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, const float *rho,
                          int g, int plan, cudaStream_t st);
    static cudaError_t next(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, float *rho,
                            float2 *u_out, int write_state, int do_scan, int apply_mask, int g, int plan,
                            cudaStream_t st);
    static cudaError_t nl_full(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                               const float *rho, int g, cudaStream_t st);
    static cudaError_t batch(int kind, const PulseTable &T, const BatchCall *C, const int2 *work, int nblocks,
                             int flag, int g, int plan, cudaStream_t st);
};

template <int NT, int PLAN>
static cudaError_t launch_nl_plan(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                                  const float *rho, int g, cudaStream_t st) {
    const size_t smem = row_smem_bytes<NT>(false);
    cudaError_t e = set_smem(k_row_nl<NT, PLAN>, smem);
    if (e != cudaSuccess) return e;
    k_row_nl<NT, PLAN><<<a.Nr, nl_threads<NT, PLAN>(), smem, st>>>(a, F32, Fb, D, rho, g);
    return cudaGetLastError();
}

template <int NT, int PLAN>
static cudaError_t launch_next_plan(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                                    float *rho, float2 *u_out, int write_state, int do_scan, int apply_mask, int g,
                                    cudaStream_t st) {
    const size_t smem = row_smem_bytes<NT>(true);
    cudaError_t e = set_smem(k_row_next<NT, PLAN>, smem);
    if (e != cudaSuccess) return e;
    k_row_next<NT, PLAN><<<a.Nr, row_threads<NT>(), smem, st>>>(a, F32, Fb, D, rho, u_out, write_state, do_scan,
                                                                apply_mask, g);
    return cudaGetLastError();
}

template <int NT>
cudaError_t RowKernels<NT>::entry(const RowFusedArgs &a, const float2 *u, float *F32, __nv_bfloat16 *Fb, float *rho,
                                  int do_scan, cudaStream_t st) {
    const size_t smem = row_smem_bytes<NT>(true);
    cudaError_t e = set_smem(k_row_entry<NT>, smem);
    if (e != cudaSuccess) return e;
    k_row_entry<NT><<<a.Nr, row_threads<NT>(), smem, st>>>(a, u, F32, Fb, rho, do_scan);
    return cudaGetLastError();
}

template <int NT>
cudaError_t RowKernels<NT>::nl(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                               const float *rho, int g, int plan, cudaStream_t st) {
    if (plan == 1 && nl_plan1_ok<NT>()) return launch_nl_plan<NT, 1>(a, F32, Fb, D, rho, g, st);
    if (plan == 2) return launch_nl_plan<NT, 2>(a, F32, Fb, D, rho, g, st);
    return launch_nl_plan<NT, 0>(a, F32, Fb, D, rho, g, st);
}

template <int NT>
cudaError_t RowKernels<NT>::next(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, float *rho,
                                 float2 *u_out, int write_state, int do_scan, int apply_mask, int g, int plan,
                                 cudaStream_t st) {
    if (plan == 1 && next_plan1_ok<NT>())
        return launch_next_plan<NT, 1>(a, F32, Fb, D, rho, u_out, write_state, do_scan, apply_mask, g, st);
    return launch_next_plan<NT, 0>(a, F32, Fb, D, rho, u_out, write_state, do_scan, apply_mask, g, st);
}

// The full-physics row kernel exists for N_t <= 4096 (three row buffers).
template <int NT>
cudaError_t RowKernels<NT>::nl_full(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                                    const float *rho, int g, cudaStream_t st) {
    if constexpr (NT > 4096) {
        return cudaErrorInvalidValue;
    } else {
        const size_t smem = full_smem_bytes<NT>();
        cudaError_t e = set_smem(k_row_nl_full<NT>, smem);
        if (e != cudaSuccess) return e;
        k_row_nl_full<NT><<<a.Nr, full_threads<NT>(), smem, st>>>(a, F32, Fb, D, rho, g);
        return cudaGetLastError();
    }
}

template <int NT>
cudaError_t RowKernels<NT>::batch(int kind, const PulseTable &T, const BatchCall *C, const int2 *work, int nblocks,
                                  int flag, int g, int plan, cudaStream_t st) {
    cudaError_t e;
    if (kind == 3) {
        if constexpr (NT > 4096) {
            return cudaErrorInvalidValue;
        } else {
            const size_t smem = full_smem_bytes<NT>();
            e = set_smem(k_row_nl_full_b<NT>, smem);
            if (e != cudaSuccess) return e;
            k_row_nl_full_b<NT><<<nblocks, full_threads<NT>(), smem, st>>>(T, C, work, g);
            return cudaGetLastError();
        }
    }
    const size_t smem = row_smem_bytes<NT>(kind != 1);
    if (kind == 0) {
        e = set_smem(k_row_entry_b<NT>, smem);
        if (e != cudaSuccess) return e;
        k_row_entry_b<NT><<<nblocks, row_threads<NT>(), smem, st>>>(T, C, work, flag);
    } else if (kind == 1) {
        if (plan == 1 && nl_plan1_ok<NT>()) {
            e = set_smem(k_row_nl_b<NT, 1>, smem);
            if (e != cudaSuccess) return e;
            k_row_nl_b<NT, 1><<<nblocks, nl_threads<NT, 1>(), smem, st>>>(T, C, work, g);
        } else if (plan == 2) {
            e = set_smem(k_row_nl_b<NT, 2>, smem);
            if (e != cudaSuccess) return e;
            k_row_nl_b<NT, 2><<<nblocks, nl_threads<NT, 2>(), smem, st>>>(T, C, work, g);
        } else {
            e = set_smem(k_row_nl_b<NT, 0>, smem);
            if (e != cudaSuccess) return e;
            k_row_nl_b<NT, 0><<<nblocks, nl_threads<NT, 0>(), smem, st>>>(T, C, work, g);
        }
    } else {
        if (plan == 1 && next_plan1_ok<NT>()) {
            e = set_smem(k_row_next_b<NT, 1>, smem);
            if (e != cudaSuccess) return e;
            k_row_next_b<NT, 1><<<nblocks, row_threads<NT>(), smem, st>>>(T, C, work, flag, g);
        } else {
            e = set_smem(k_row_next_b<NT, 0>, smem);
            if (e != cudaSuccess) return e;
            k_row_next_b<NT, 0><<<nblocks, row_threads<NT>(), smem, st>>>(T, C, work, flag, g);
        }
    }
    return cudaGetLastError();
}

// Instantiated in k_row_n*.cu.
#define NLSE_ROW_EXTERN(X)                  \
    X(16) X(32) X(64) X(128) X(256) X(512)  \
    X(1024) X(2048) X(4096) X(8192)
#define NLSE_ROW_DECLARE_EXTERN(n) extern template struct RowKernels<n>;
NLSE_ROW_EXTERN(NLSE_ROW_DECLARE_EXTERN)
