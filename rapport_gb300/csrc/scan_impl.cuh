// Newton-linearised parallel scan of the carrier-rate march, shared by the
// standalone scan kernel and the fused row kernels.  (Derivation in k_scan.cu.)
#pragma once
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
__device__ __forceinline__ float lut_rate_dt(float I, const float *__restrict__ lut, const ScanParams &p) {
    if (!isfinite(I) || I < 0.0f) I = 0.0f;
    I = fminf(fmaxf(I, p.Imin), p.Imax);
    float pos = (log10f(I) - p.lut_log_min) * p.lut_inv_dlog;
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
    float e = expf(z);
    float em1 = expm1f(z);
    float az = fabsf(z);
    float ph = az > 1e-4f ? em1 / z : fmaf(z, fmaf(z, fmaf(z, 1.0f / 24.0f, 1.0f / 6.0f), 0.5f), 1.0f);
    float y = fmaf(e, x, b * d * ph);
    float dd = (x >= p.x_tiny && x < p.na) ? -p.inv_na : 0.0f;
    float dph;  // phi1'(z) = (z e^z - (e^z - 1)) / z^2
    if (az < 0.1f)
        dph = fmaf(z, fmaf(z, fmaf(z, fmaf(z, fmaf(z, 1.0f / 840.0f, 1.0f / 144.0f), 1.0f / 30.0f),
                                   0.125f), 1.0f / 3.0f), 0.5f);
    else
        dph = (z * e - em1) / (z * z);
    float zp = a * dd;
    float Jv = fmaf(x * e, zp, e) + b * fmaf(dd, ph, d * dph * zp);
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


// Solve one row's carrier march (all threads of the CTA).  On entry sI[0..Nt)
// holds the intensities (synced); sW, sx, sJ, sB are scratch of Nt floats
// each (may alias any other buffer the caller no longer needs).  On return
// (synced) sx[t] holds the densities, sx[0] = x0.
// Shared-memory slot of step n when thread t owns the contiguous chunk
// [t C, (t + 1) C): slot j T + t for n = t C + j -- the threads of a warp then
// touch consecutive words at every j (a plain layout would be C-way conflicted).
__device__ __forceinline__ int scan_slot(int n, int C) { return (n % C) * (int)blockDim.x + n / C; }

// Number of floats each scan array needs for Nt points with `threads` threads:
// one past the largest slot, reached at remainder C - 1 (= Nt for powers of two).
__host__ __device__ __forceinline__ constexpr int scan_span(int Nt, int threads) {
    return ((Nt - 1 + threads - 1) / threads - 1) * threads +
           (Nt - (Nt - 1 + threads - 1) / threads) / ((Nt - 1 + threads - 1) / threads) + 1;
}

// Solve one row's carrier march (all threads of the CTA).  On entry sI holds
// the intensities at slots scan_slot(t, C) (synced); sW, sx, sJ, sB are
// scratch of scan_span(Nt) floats each (may alias any other buffer the caller
// no longer needs).  On return (synced) sx[scan_slot(t, C)] holds the density
// at t, sx[slot 0] = x0.  C = chunk of steps per thread = ceil((Nt-1)/blockDim).
static __device__ void scan_row(const float *sI, float *sW, float *sx, float *sJ, float *sB, int Nt,
                                const ScanParams &p, const float *__restrict__ lut, float x0, int *stats) {
    __shared__ Aff wsum[32];
    __shared__ float red[100];
    const int T = Nt - 1;
    const int C = (T + blockDim.x - 1) / blockDim.x;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) {
        const int q = scan_slot(t, C);
        sW[q] = lut_rate_dt(sI[q], lut, p);
        sx[q] = t == 0 ? x0 : 0.0f;
    }
    __syncthreads();
    const int n0 = min((int)threadIdx.x * C, T), n1 = min(n0 + C, T);
    int converged = 0, clamp_any = 0;
    for (int it = 0; it < SCAN_MAX_IT; ++it) {
        Aff acc{1.0f, 0.0f};
        bool cl = false;
        for (int n = n0; n < n1; ++n) {
            const int q0 = scan_slot(n, C), q1 = scan_slot(n + 1, C);
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
        for (int n = n0; n < n1; ++n) {
            const int q0 = scan_slot(n, C), q1 = scan_slot(n + 1, C);
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
                const int q0 = scan_slot(n, C), q1 = scan_slot(n + 1, C);
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
