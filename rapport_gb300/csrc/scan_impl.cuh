// Newton-linearised parallel scan of the carrier-rate march, shared by the
// standalone scan kernel and the fused row kernels.  (Derivation in k_scan.cu.)
#pragma once
#include <float.h>

#include "nlse_internal.cuh"


#define SCAN_MAX_IT 16
#define SCAN_TOL 1e-6f

struct Aff {
    float A, B;  // x -> A x + B
};

// apply `first`, then `second`
__device__ __forceinline__ Aff aff_then(Aff first, Aff second) {
    return Aff{second.A * first.A, fmaf(second.A, first.B, second.B)};
}

// W(I) * dt, linear in log10 I on the uniform table (kernels.py:14-26).
// I_zero: below it the table's entries on both sides are zero and so is the
// result, without the logarithm and the table reads.
__device__ __forceinline__ float lut_rate_dt(float I, const float *__restrict__ lut, float I_zero,
                                             const ScanParams &p) {
    if (!isfinite(I) || I < 0.0f) I = 0.0f;
    if (I < I_zero) return 0.0f;
    I = fminf(fmaxf(I, p.Imin), p.Imax);
    // log10 from the hardware log2 (~2^-22 relative): it moves the interpolation
    // weight by ~1e-5 of one of the table's 0.004-decade intervals
    float pos = fmaf(__log2f(I), 0.301029995663981f, -p.lut_log_min) * p.lut_inv_dlog;
    int k = (int)pos;
    k = min(max(k, 0), p.lut_n - 2);
    float w0 = __ldg(&lut[k]), w1 = __ldg(&lut[k + 1]);
    float w = fmaf(pos - (float)k, w1 - w0, w0);
    return (isfinite(w) && w >= 0.0f) ? w : 0.0f;
}

// One step of the march and its derivative d f / d x.
__device__ __forceinline__ float step_map(float x, float a, float b, const ScanParams &p, float *J,
                                          bool *clamped) {
    // (na - x) is exact near saturation, so d is exactly 0 at x = na as in FP64;
    // below x_tiny the FP32 depletion factor is exactly 1 (and constant)
    float d = x < p.x_tiny ? 1.0f : fminf(fmaxf((p.na - x) * p.inv_na, 0.0f), 1.0f);
    float z = fmaf(a, d, -p.c_rec);
    if (z > 80.0f) {
        // e^z overflows FP32 but not FP64 (below z = 709.78): there the reference
        // computes y = e^z x + b d (e^z - 1)/z, which exceeds na unless x and b d
        // are tiny -- evaluate it in log space; beyond 709.78 FP64 overflows too
        // and the reference's non-finite -> 0 rule resets the density.
        *J = 0.0f;
        if (z > 709.78f) return 0.0f;
        float s = fmaf(b * d, 1.0f / z, x);
        if (!(s > 0.0f)) return 0.0f;
        float lg = z + logf(s);
        if (lg > logf(p.na)) {
            *clamped = true;
            return p.na;
        }
        return expf(lg);
    }
    // z >= -dt/tau_rec here (a, d >= 0); e^z as 1 + expm1(z) where that is exact
    // to the last bit's rounding (z > -1/2), phi1(z) = expm1(z) / z by its series
    // where the fifth-order truncation is below 1e-11 (|z| < 0.05)
    float em1 = expm1f(z);
    float e = z > -0.5f ? 1.0f + em1 : expf(z);
    float az = fabsf(z);
    float ph = az >= 0.05f ? __fdividef(em1, z)
                           : fmaf(z, fmaf(z, fmaf(z, fmaf(z, fmaf(z, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f),
                                                  1.0f / 6.0f), 0.5f), 1.0f);
    // e^z x + b d phi1(z) as x + (expm1(z) x + b d phi1(z)): the decay factor's
    // rounding then scales only the change, not x, so it does not bias the
    // density the same way at every one of the row's steps
    float y = x + fmaf(em1, x, b * d * ph);
    float dd = (x >= p.x_tiny && x < p.na) ? -p.inv_na : 0.0f;
    float dph;  // phi1'(z) = (z e^z - (e^z - 1)) / z^2
    if (az < 0.1f)
        dph = fmaf(z, fmaf(z, fmaf(z, fmaf(z, fmaf(z, 1.0f / 840.0f, 1.0f / 144.0f), 1.0f / 30.0f),
                                   0.125f), 1.0f / 3.0f), 0.5f);
    else
        dph = __fdividef(fmaf(z, e, -em1), z * z);
    float zp = a * dd;
    float Jv = fmaf(b, fmaf(dd, ph, d * dph * zp), fmaf(x * e, zp, e));
    if (!isfinite(Jv)) Jv = 0.0f;
    if (!isfinite(y) || y < 0.0f) {
        y = 0.0f;
        Jv = 0.0f;
    } else if (y > p.na) {
        y = p.na;
        Jv = 0.0f;
        *clamped = true;
    }
    *J = Jv;
    return y;
}

static __device__ Aff block_exclusive_scan(Aff v, Aff *wsum) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    Aff inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        float A = __shfl_up_sync(0xffffffffu, inc.A, off);
        float B = __shfl_up_sync(0xffffffffu, inc.B, off);
        if (lane >= off) inc = aff_then(Aff{A, B}, inc);
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        Aff w = lane < nw ? wsum[lane] : Aff{1.0f, 0.0f};
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            float A = __shfl_up_sync(0xffffffffu, w.A, off);
            float B = __shfl_up_sync(0xffffffffu, w.B, off);
            if (lane >= off) w = aff_then(Aff{A, B}, w);
        }
        wsum[lane] = w;
    }
    __syncthreads();
    Aff wpre = wid > 0 ? wsum[wid - 1] : Aff{1.0f, 0.0f};
    float A = __shfl_up_sync(0xffffffffu, inc.A, 1);
    float B = __shfl_up_sync(0xffffffffu, inc.B, 1);
    Aff lex = lane > 0 ? Aff{A, B} : Aff{1.0f, 0.0f};
    Aff r = aff_then(wpre, lex);
    __syncthreads();
    return r;
}

// Block-wide max of two floats and OR of a flag; result broadcast to all threads.
static __device__ void block_reduce(float &m1, float &m2, int &f, float *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, off));
        m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, off));
        f |= __shfl_xor_sync(0xffffffffu, f, off);
    }
    if (lane == 0) {
        red[wid] = m1;
        red[32 + wid] = m2;
        red[64 + wid] = __int_as_float(f);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = red[0], b = red[32];
        int c = __float_as_int(red[64]);
        for (int w = 1; w < nw; ++w) {
            a = fmaxf(a, red[w]);
            b = fmaxf(b, red[32 + w]);
            c |= __float_as_int(red[64 + w]);
        }
        red[96] = a;
        red[97] = b;
        red[98] = __int_as_float(c);
    }
    __syncthreads();
    m1 = red[96];
    m2 = red[97];
    f = __float_as_int(red[98]);
    __syncthreads();
}


// Shared-memory slot of step n when thread t owns the contiguous chunk
// [t C, (t + 1) C): slot j (T + pad) + t for n = t C + j.  In the sweeps the
// threads of a warp touch consecutive words at every j; in the loops where
// consecutive threads take consecutive n (filling the intensities, reading
// the densities out), n % C spreads the lanes over C rows whose stride
// T + pad is (32 / C) banks apart mod 32, so those are conflict-free too
// (without the pad they would be C-way conflicted).
__host__ __device__ __forceinline__ constexpr int scan_pad(int C) { return C >= 32 ? 1 : 32 / C; }

// C = ceil((Nt - 1) / T) is a power of two for power-of-two Nt and T = 256,
// so the slot map is two masks / shifts; S = T + pad is the row stride.
struct ScanLayout {
    int C, logC, S;
};

__device__ __forceinline__ ScanLayout scan_layout(int Nt) {
    const int C = (Nt - 1 + (int)blockDim.x - 1) / (int)blockDim.x;
    return ScanLayout{C, 31 - __clz(C), (int)blockDim.x + scan_pad(C)};
}

__device__ __forceinline__ int scan_slot(int n, const ScanLayout &L) {
    return (n & (L.C - 1)) * L.S + (n >> L.logC);
}

// Number of floats each scan array needs for Nt points with `threads` threads:
// one past the largest slot, reached at n = Nt - 1 (remainder C - 1 for powers of two).
__host__ __device__ __forceinline__ constexpr int scan_span(int Nt, int threads) {
    return ((Nt - 1 + threads - 1) / threads - 1) * (threads + scan_pad((Nt - 1 + threads - 1) / threads)) +
           (Nt - 1) / ((Nt - 1 + threads - 1) / threads) + 1;
}

// Solve one row's carrier march (all threads of the CTA).  On entry sI holds
// the intensities at slots scan_slot(t, scan_layout(Nt)) (synced); sW, sx, sJ,
// sB are scratch of scan_span(Nt) floats each (may alias any other buffer the
// caller no longer needs).  On return (synced) sx[slot of t] holds the density
// at t, sx[slot 0] = x0.  C = chunk of steps per thread = ceil((Nt-1)/blockDim).
// Whether a point keeps a row's march from being skipped.  With x0 = 0 and
// W = 0 at every point, every step maps 0 to exactly 0 (y = 0 + e^z 0 + 0),
// every affine map has B = +0 and the row's densities are +0 -- provided the
// products of the maps' A = e^z stay finite, which (Nt - 1) a_coef I < 64 at
// every point guarantees (z <= a_coef I_avg).  Such a row (most rows, away
// from the beam) skips the sweeps; the result is the same bit for bit.
__device__ __forceinline__ int march_needed(float W, float I, int Nt, const ScanParams &p) {
    return W != 0.0f || !((float)(Nt - 1) * (p.a_coef * I) < 64.0f);
}

static __device__ void scan_row(const float *sI, float *sW, float *sx, float *sJ, float *sB, int Nt,
                                const ScanParams &p, const float *__restrict__ lut, float x0, int *stats) {
    __shared__ Aff wsum[32];
    __shared__ float red[100];
    const int T = Nt - 1;
    const ScanLayout L = scan_layout(Nt);
    const int C = L.C;
    int need = 0;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        const int q = scan_slot(t, L);
        sW[q] = lut_rate_dt(sI[q], lut, p.I_w0, p);
        sx[q] = t == 0 ? x0 : 0.0f;
        need |= march_needed(sW[q], sI[q], Nt, p);
    }
    // a row without ionisation and carriers stays at exactly zero (see march_needed)
    if (!__syncthreads_or(need) && x0 == 0.0f) return;
    // the thread's chunk: steps n0 .. n1-1 at slots j S + tid; the step after
    // the chunk's last is the next thread's first (slot tid + 1)
    const int n0 = min((int)threadIdx.x * C, T), n1 = min(n0 + C, T);
    const int q_last = (int)threadIdx.x + 1;
    int converged = 0, clamp_any = 0;
    for (int it = 0; it < SCAN_MAX_IT; ++it) {
        Aff acc{1.0f, 0.0f};
        bool cl = false;
        for (int n = n0, q0 = threadIdx.x; n < n1; ++n, q0 += L.S) {
            const int q1 = n + 1 - n0 < C ? q0 + L.S : q_last;
            float Ia = 0.5f * (sI[q0] + sI[q1]);
            float b = 0.5f * (sW[q0] + sW[q1]);
            float xn = sx[q0];
            float J = 0.0f, F = 0.0f;
            if (isfinite(Ia)) F = step_map(xn, p.a_coef * Ia, b, p, &J, &cl);
            float Bv = fmaf(-J, xn, F);
            sJ[q0] = J;
            sB[q0] = Bv;
            acc = aff_then(acc, Aff{J, Bv});
        }
        Aff pre = block_exclusive_scan(acc, wsum);
        float xs = fmaf(pre.A, x0, pre.B);
        float dmax = 0.0f, xmax = 0.0f;
        for (int n = n0, q0 = threadIdx.x; n < n1; ++n, q0 += L.S) {
            const int q1 = n + 1 - n0 < C ? q0 + L.S : q_last;
            xs = fmaf(sJ[q0], xs, sB[q0]);
            dmax = fmaxf(dmax, fabsf(xs - sx[q1]));
            xmax = fmaxf(xmax, fabsf(xs));
            sx[q1] = xs;
        }
        int f = cl ? 1 : 0;
        block_reduce(dmax, xmax, f, red);
        clamp_any |= f;
        if (clamp_any) break;
        // The first sweep starts from x = 0, where the depletion is frozen at
        // d = 1 (J = e^z, B = b phi1(z)): if the whole solution stays below
        // x_tiny the map is exactly that affine map, so the sweep is exact.
        if (dmax <= SCAN_TOL * xmax || (it == 0 && xmax < p.x_tiny)) {
            converged = 1;
            break;
        }
    }
    if (!converged) {
        // exact sequential march (saturated or non-converging row)
        if (threadIdx.x == 0) {
            float x = x0;
            bool cl = false;
            for (int n = 0; n < T; ++n) {
                const int q0 = scan_slot(n, L), q1 = scan_slot(n + 1, L);
                float Ia = 0.5f * (sI[q0] + sI[q1]);
                float b = 0.5f * (sW[q0] + sW[q1]);
                float J;
                x = isfinite(Ia) ? step_map(x, p.a_coef * Ia, b, p, &J, &cl) : 0.0f;
                sx[q1] = x;
            }
            if (stats) atomicAdd(&stats[1], 1);
        }
    }
    __syncthreads();
}

// The scan layout of an NT-point row marched by T threads, at compile time
// (the fused row kernels know both): C steps per thread, row stride S.
template <int NT, int T>
struct ScanShape {
    static constexpr int C = (NT - 1 + T - 1) / T;
    static constexpr int logC = C >= 16 ? 4 : (C >= 8 ? 3 : (C >= 4 ? 2 : (C >= 2 ? 1 : 0)));
    static constexpr int S = T + scan_pad(C);
    static_assert((1 << logC) == C, "C is a power of two for power-of-two NT and T");
    __device__ __forceinline__ static int slot(int n) { return (n & (C - 1)) * S + (n >> logC); }
};

// scan_row for an NT-point row and T = blockDim.x threads known at compile
// time: the same iterations, step maps and roundings (results are identical),
// with the thread's C steps unrolled -- the slots are constant offsets, each
// step's right-hand intensity, rate and iterate are the next step's left-hand
// ones, and the affine maps of the sweep stay in registers between the scan
// and the update instead of passing through shared memory.
template <int NT, int T>
static __device__ void scan_row_ct(const float *sI, float *sW, float *sx, const ScanParams &p,
                                   const float *__restrict__ lut, float x0, int *stats) {
    using Sh = ScanShape<NT, T>;
    constexpr int C = Sh::C, S = Sh::S;
    __shared__ Aff wsum[32];
    __shared__ float red[100];
    const int tid = threadIdx.x;
    int need = 0;
    for (int t = tid; t < NT; t += T) {
        const int q = Sh::slot(t);
        const float w = lut_rate_dt(sI[q], lut, p.I_w0, p);
        sW[q] = w;
        sx[q] = t == 0 ? x0 : 0.0f;
        need |= march_needed(w, sI[q], NT, p);
    }
    // a row without ionisation and carriers stays at exactly zero (see march_needed)
    if (!__syncthreads_or(need) && x0 == 0.0f) return;
    // the thread's steps n0 .. n0 + nst - 1 at slots j S + tid; the step after
    // its last is the next thread's first (slot tid + 1)
    const int n0 = min(tid * C, NT - 1), nst = min(n0 + C, NT - 1) - n0;
    int converged = 0, clamp_any = 0;
    for (int it = 0; it < SCAN_MAX_IT; ++it) {
        float J[C], B[C];
        Aff acc{1.0f, 0.0f};
        bool cl = false;
        float I0 = 0.0f, W0 = 0.0f, xn = 0.0f;
        if (nst > 0) {
            I0 = sI[tid];
            W0 = sW[tid];
            xn = sx[tid];
        }
#pragma unroll
        for (int j = 0; j < C; ++j) {
            if (j < nst) {
                const int q1 = j + 1 < C ? (j + 1) * S + tid : tid + 1;
                const float I1 = sI[q1], W1 = sW[q1];
                float Ia = 0.5f * (I0 + I1);
                float b = 0.5f * (W0 + W1);
                float Jv = 0.0f, F = 0.0f;
                if (isfinite(Ia)) F = step_map(xn, p.a_coef * Ia, b, p, &Jv, &cl);
                const float Bv = fmaf(-Jv, xn, F);
                J[j] = Jv;
                B[j] = Bv;
                acc = aff_then(acc, Aff{Jv, Bv});
                I0 = I1;
                W0 = W1;
                xn = sx[q1];
            }
        }
        Aff pre = block_exclusive_scan(acc, wsum);
        float xs = fmaf(pre.A, x0, pre.B);
        float dmax = 0.0f, xmax = 0.0f;
#pragma unroll
        for (int j = 0; j < C; ++j) {
            if (j < nst) {
                const int q1 = j + 1 < C ? (j + 1) * S + tid : tid + 1;
                xs = fmaf(J[j], xs, B[j]);
                dmax = fmaxf(dmax, fabsf(xs - sx[q1]));
                xmax = fmaxf(xmax, fabsf(xs));
                sx[q1] = xs;
            }
        }
        int f = cl ? 1 : 0;
        block_reduce(dmax, xmax, f, red);
        clamp_any |= f;
        if (clamp_any) break;
        if (dmax <= SCAN_TOL * xmax || (it == 0 && xmax < p.x_tiny)) {
            converged = 1;
            break;
        }
    }
    if (!converged) {
        // exact sequential march (saturated or non-converging row)
        if (tid == 0) {
            float x = x0;
            bool cl = false;
            for (int n = 0; n < NT - 1; ++n) {
                const int q0 = Sh::slot(n), q1 = Sh::slot(n + 1);
                float Ia = 0.5f * (sI[q0] + sI[q1]);
                float b = 0.5f * (sW[q0] + sW[q1]);
                float Jv;
                x = isfinite(Ia) ? step_map(x, p.a_coef * Ia, b, p, &Jv, &cl) : 0.0f;
                sx[q1] = x;
            }
            if (stats) atomicAdd(&stats[1], 1);
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------------ two populations (self-trapped excitons)
// With the exciton channel on, the reference march (kernels.py:72-95) advances
// (e, s) = (rho_e, rho_s) by
//   e' = e^{ze} e + qe phi1(ze),  ze = a d - c,            qe = b d + r s / na
//   s' = e^{zs} s + qs phi1(zs),  zs = -r / na - cs,       qs = c e
// with d = depletion(e), r = bs + as e (re-ionisation), a = beta_g dt I_avg,
// as = beta_s dt I_avg, b / bs = dt W_avg / dt Ws_avg, c = dt / tau_r,
// cs = dt / tau_ste; each population's non-finite/negative result -> 0, and
// e' + s' > na rescales both.  Newton's method linearises the map into a 2x2
// affine recurrence, solved by a block scan of (matrix, vector) pairs.
struct Aff2 {
    float m00, m01, m10, m11, v0, v1;  // x -> M x + v
};

__device__ __forceinline__ Aff2 aff2_then(const Aff2 &f, const Aff2 &g) {  // f first, then g
    Aff2 r;
    r.m00 = fmaf(g.m00, f.m00, g.m01 * f.m10);
    r.m01 = fmaf(g.m00, f.m01, g.m01 * f.m11);
    r.m10 = fmaf(g.m10, f.m00, g.m11 * f.m10);
    r.m11 = fmaf(g.m10, f.m01, g.m11 * f.m11);
    r.v0 = fmaf(g.m00, f.v0, fmaf(g.m01, f.v1, g.v0));
    r.v1 = fmaf(g.m10, f.v0, fmaf(g.m11, f.v1, g.v1));
    return r;
}

__device__ __forceinline__ Aff2 aff2_identity() { return Aff2{1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f}; }

// phi1(z) and phi1'(z), accurate for small |z|
__device__ __forceinline__ void phi1_d(float z, float e, float em1, float *ph, float *dph) {
    const float az = fabsf(z);
    *ph = az > 1e-4f ? em1 / z : fmaf(z, fmaf(z, fmaf(z, 1.0f / 24.0f, 1.0f / 6.0f), 0.5f), 1.0f);
    *dph = az < 0.1f ? fmaf(z, fmaf(z, fmaf(z, fmaf(z, fmaf(z, 1.0f / 840.0f, 1.0f / 144.0f), 1.0f / 30.0f), 0.125f),
                                    1.0f / 3.0f), 0.5f)
                     : fmaf(z, e, -em1) / (z * z);
}

// One step of the two-population march and its Jacobian; sets *clamped when
// the e + s <= na rescale fires or e^{ze} leaves the FP32 range (ze > 80):
// the caller then re-marches sequentially with step_exact2.  s / na is formed
// first: r s alone overflows FP32 once both densities pass ~1e19.
__device__ __forceinline__ void step_map2(float e, float s, float a, float as, float b, float bs, const ScanParams &p,
                                          float *eo, float *so, Aff2 *J, bool *clamped) {
    const float d = e < p.x_tiny ? 1.0f : fminf(fmaxf((p.na - e) * p.inv_na, 0.0f), 1.0f);
    const float dd = (e >= p.x_tiny && e < p.na) ? -p.inv_na : 0.0f;
    const float r = fmaf(as, e, bs);
    const float ze = fmaf(a, d, -p.c_rec), zs = fmaf(-r, p.inv_na, -p.cs_ste);
    if (ze > 80.0f) *clamped = true;
    const float ee = expf(ze), eem1 = expm1f(ze), es = expf(zs), esm1 = expm1f(zs);
    float phe, dphe, phs, dphs;
    phi1_d(ze, ee, eem1, &phe, &dphe);
    phi1_d(zs, es, esm1, &phs, &dphs);
    const float sn = s * p.inv_na;
    const float qe = fmaf(b, d, r * sn), qs = p.c_rec * e;
    float y0 = e + fmaf(eem1, e, qe * phe);
    float y1 = s + fmaf(esm1, s, qs * phs);
    const float ze_e = a * dd, zs_e = -as * p.inv_na;
    const float qe_e = fmaf(b, dd, as * sn), qe_s = r * p.inv_na;
    Aff2 j;
    j.m00 = fmaf(ee, fmaf(e, ze_e, 1.0f), fmaf(qe_e, phe, qe * dphe * ze_e));
    j.m01 = qe_s * phe;
    j.m10 = fmaf(es * s, zs_e, fmaf(p.c_rec, phs, qs * dphs * zs_e));
    j.m11 = es;
    if (!isfinite(j.m00) || !isfinite(j.m01)) j.m00 = j.m01 = 0.0f;
    if (!isfinite(j.m10) || !isfinite(j.m11)) j.m10 = j.m11 = 0.0f;
    if (!isfinite(y0) || y0 < 0.0f) {
        y0 = 0.0f;
        j.m00 = j.m01 = 0.0f;
    }
    if (!isfinite(y1) || y1 < 0.0f) {
        y1 = 0.0f;
        j.m10 = j.m11 = 0.0f;
    }
    if (y0 + y1 > p.na) *clamped = true;
    *eo = y0;
    *so = y1;
    *J = j;
}

// The reference's two-population step in FP32 (sequential).  Where e^{ze}
// overflows FP32 but not FP64 (80 < ze <= 709.78) the electron update
// e' = e^{ze} (e + qe/ze) - qe/ze is taken in log space; when it exceeds na the
// reference's rescale by na / (e' + s') is applied in that form too, which
// leaves s' = na s' / (e' + s') tiny but resolved.  Beyond 709.78 FP64
// overflows as well and the non-finite -> 0 rule resets e'.
__device__ __forceinline__ void step_exact2(float &e, float &s, float Ia, float b, float bs, const ScanParams &p) {
    if (!isfinite(Ia)) {
        e = s = 0.0f;
        return;
    }
    const float a = p.a_coef * Ia, as = p.as_coef * Ia;
    const float d = e < p.x_tiny ? 1.0f : fminf(fmaxf((p.na - e) * p.inv_na, 0.0f), 1.0f);
    const float r = fmaf(as, e, bs);
    const float ze = fmaf(a, d, -p.c_rec), zs = fmaf(-r, p.inv_na, -p.cs_ste);
    const float qe = fmaf(b, d, r * (s * p.inv_na)), qs = p.c_rec * e;
    float ph, dph;
    const float es = expf(zs);
    phi1_d(zs, es, expm1f(zs), &ph, &dph);
    float y1 = fmaf(es, s, qs * ph);
    if (!isfinite(y1) || y1 < 0.0f) y1 = 0.0f;
    float y0;
    if (ze > 709.78f) {
        y0 = 0.0f;
    } else if (ze > 80.0f) {
        const float c0 = qe / ze, sm = e + c0;
        if (!(sm > 0.0f) || !isfinite(sm)) {
            y0 = 0.0f;
        } else {
            const float lg = ze + logf(sm);
            if (lg > logf(p.na)) {
                const float w = y1 > 0.0f ? expf(logf(y1) - lg) : 0.0f;  // s' / e' before the rescale
                const float k = p.na / (1.0f + w);
                e = k;
                s = k * w;
                return;
            }
            y0 = expf(lg) - c0;
        }
    } else {
        const float ee = expf(ze);
        phi1_d(ze, ee, expm1f(ze), &ph, &dph);
        y0 = fmaf(ee, e, qe * ph);
        if (!isfinite(y0) || y0 < 0.0f) y0 = 0.0f;
    }
    if (y0 + y1 > p.na) {
        const float k = p.na / (y0 + y1);
        y0 *= k;
        y1 *= k;
    }
    e = y0;
    s = y1;
}

static __device__ Aff2 block_exclusive_scan2(Aff2 v, Aff2 *wsum) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    Aff2 inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        Aff2 o;
        o.m00 = __shfl_up_sync(0xffffffffu, inc.m00, off);
        o.m01 = __shfl_up_sync(0xffffffffu, inc.m01, off);
        o.m10 = __shfl_up_sync(0xffffffffu, inc.m10, off);
        o.m11 = __shfl_up_sync(0xffffffffu, inc.m11, off);
        o.v0 = __shfl_up_sync(0xffffffffu, inc.v0, off);
        o.v1 = __shfl_up_sync(0xffffffffu, inc.v1, off);
        if (lane >= off) inc = aff2_then(o, inc);
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        Aff2 w = lane < nw ? wsum[lane] : aff2_identity();
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            Aff2 o;
            o.m00 = __shfl_up_sync(0xffffffffu, w.m00, off);
            o.m01 = __shfl_up_sync(0xffffffffu, w.m01, off);
            o.m10 = __shfl_up_sync(0xffffffffu, w.m10, off);
            o.m11 = __shfl_up_sync(0xffffffffu, w.m11, off);
            o.v0 = __shfl_up_sync(0xffffffffu, w.v0, off);
            o.v1 = __shfl_up_sync(0xffffffffu, w.v1, off);
            if (lane >= off) w = aff2_then(o, w);
        }
        wsum[lane] = w;
    }
    __syncthreads();
    const Aff2 wpre = wid > 0 ? wsum[wid - 1] : aff2_identity();
    Aff2 lex;
    lex.m00 = __shfl_up_sync(0xffffffffu, inc.m00, 1);
    lex.m01 = __shfl_up_sync(0xffffffffu, inc.m01, 1);
    lex.m10 = __shfl_up_sync(0xffffffffu, inc.m10, 1);
    lex.m11 = __shfl_up_sync(0xffffffffu, inc.m11, 1);
    lex.v0 = __shfl_up_sync(0xffffffffu, inc.v0, 1);
    lex.v1 = __shfl_up_sync(0xffffffffu, inc.v1, 1);
    if (lane == 0) lex = aff2_identity();
    const Aff2 r = aff2_then(wpre, lex);
    __syncthreads();
    return r;
}

// Two-population march of one row (all threads).  sI: intensities at slots
// (synced); scratch arrays of scan_span(Nt) floats: sW, sWs, se, ss, and J
// (4 arrays jm[0..3]) + B (2 arrays jb[0..1]).  On return (synced) se / ss hold
// rho_e / rho_s at the slots.  x0e / x0s: the t = 0 values.
static __device__ void scan_row2(const float *sI, float *sW, float *sWs, float *se, float *ss, float *const *jm,
                                 float *const *jb, int Nt, const ScanParams &p, const float *__restrict__ lut,
                                 const float *__restrict__ lut_s, float x0e, float x0s, int *stats) {
    __shared__ Aff2 wsum[32];
    __shared__ float red[100];
    const int T = Nt - 1;
    const ScanLayout L = scan_layout(Nt);
    const int C = L.C;
    int need = 0;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        const int q = scan_slot(t, L);
        sW[q] = lut_rate_dt(sI[q], lut, p.I_w0, p);
        sWs[q] = lut_rate_dt(sI[q], lut_s, p.I_w0s, p);
        se[q] = t == 0 ? x0e : 0.0f;
        ss[q] = t == 0 ? x0s : 0.0f;
        need |= march_needed(sW[q], sI[q], Nt, p) || sWs[q] != 0.0f;
    }
    // As for one population: with both rates zero along the row and both
    // densities starting at zero, every step maps (0, 0) to exactly (0, 0)
    // (the re-ionisation and the exciton source vanish with the densities),
    // the affine offsets stay +0 and the maps' products finite: the row stays
    // at zero and skips the sweeps.
    if (!__syncthreads_or(need) && x0e == 0.0f && x0s == 0.0f) return;
    const int n0 = min((int)threadIdx.x * C, T), n1 = min(n0 + C, T);
    const int q_last = (int)threadIdx.x + 1;
    int converged = 0, clamp_any = 0;
    for (int it = 0; it < SCAN_MAX_IT; ++it) {
        Aff2 acc = aff2_identity();
        bool cl = false;
        for (int n = n0, q0 = threadIdx.x; n < n1; ++n, q0 += L.S) {
            const int q1 = n + 1 - n0 < C ? q0 + L.S : q_last;
            const float Ia = 0.5f * (sI[q0] + sI[q1]);
            const float b = 0.5f * (sW[q0] + sW[q1]), bs = 0.5f * (sWs[q0] + sWs[q1]);
            const float e = se[q0], s = ss[q0];
            Aff2 J = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            float eo = 0.0f, so = 0.0f;
            if (isfinite(Ia)) step_map2(e, s, p.a_coef * Ia, p.as_coef * Ia, b, bs, p, &eo, &so, &J, &cl);
            J.v0 = eo - fmaf(J.m00, e, J.m01 * s);
            J.v1 = so - fmaf(J.m10, e, J.m11 * s);
            jm[0][q0] = J.m00;
            jm[1][q0] = J.m01;
            jm[2][q0] = J.m10;
            jm[3][q0] = J.m11;
            jb[0][q0] = J.v0;
            jb[1][q0] = J.v1;
            acc = aff2_then(acc, J);
        }
        const Aff2 pre = block_exclusive_scan2(acc, wsum);
        float xe = fmaf(pre.m00, x0e, fmaf(pre.m01, x0s, pre.v0));
        float xs = fmaf(pre.m10, x0e, fmaf(pre.m11, x0s, pre.v1));
        float dmax = 0.0f, xmax = 0.0f;
        for (int n = n0, q0 = threadIdx.x; n < n1; ++n, q0 += L.S) {
            const int q1 = n + 1 - n0 < C ? q0 + L.S : q_last;
            const float ne = fmaf(jm[0][q0], xe, fmaf(jm[1][q0], xs, jb[0][q0]));
            const float ns = fmaf(jm[2][q0], xe, fmaf(jm[3][q0], xs, jb[1][q0]));
            xe = ne;
            xs = ns;
            dmax = fmaxf(dmax, fmaxf(fabsf(xe - se[q1]), fabsf(xs - ss[q1])));
            xmax = fmaxf(xmax, fmaxf(fabsf(xe), fabsf(xs)));
            se[q1] = xe;
            ss[q1] = xs;
        }
        int f = cl ? 1 : 0;
        block_reduce(dmax, xmax, f, red);
        clamp_any |= f;
        if (clamp_any) break;
        // converged: the sweep changed nothing by more than 1e-6 of the row's
        // largest density, or by less than the smallest normal FP32 number --
        // at the rim of the ionised region the densities can be ~1e-38 cm^-3,
        // where the iterates settle into denormal rounding noise tens of ulps
        // wide and never meet a relative test (the row would otherwise be
        // re-marched sequentially by one thread)
        if (it > 0 && (dmax <= SCAN_TOL * xmax || dmax <= FLT_MIN)) {
            converged = 1;
            break;
        }
    }
    if (!converged) {
        if (threadIdx.x == 0) {
            float e = x0e, s = x0s;
            for (int n = 0; n < T; ++n) {
                const int q0 = scan_slot(n, L), q1 = scan_slot(n + 1, L);
                step_exact2(e, s, 0.5f * (sI[q0] + sI[q1]), 0.5f * (sW[q0] + sW[q1]), 0.5f * (sWs[q0] + sWs[q1]), p);
                se[q1] = e;
                ss[q1] = s;
            }
            if (stats) atomicAdd(&stats[1], 1);
        }
    }
    __syncthreads();
}
