// Full-physics nonlinear block: split() with Raman, self-steepening and
// space-time focusing (operators.py:89-146, grids.py:79-116), one row of the
// field per CTA, every transform in shared memory.
//
// split(S) of the reference, for a row S(t):
//   kerr_I = (1 - f_R) |S|^2 [instantaneous] + f_R Re F^-1[F[|S|^2] R_f] [Raman]
//   X1 = i kerr_pref kerr_I S,   X2 = photo S,
//   X3 = (-pp_abs rho + i (-pp_def rho + ste_pref rho_s)) S
//   k  = F^-1[(T^2 F[X1] - T F[X2] + F[X3]) U^-1] + alpha S
// with T = 1 without self-steepening and U^-1 = 1 without space-time focusing.
// Transforms a term does not need are skipped: with U^-1 = 1, X3 is added
// pointwise; with T = U^-1 = 1 the whole right-hand side is pointwise (the
// algebraically reduced form of nl_rhs, with the Raman-convolved intensity).
// The reference then zeroes k where |S|^2 < 1e-30 and every non-finite k
// (nan_to_num).  Because every term of the row passes through FFTs there, one
// non-finite X anywhere in the row makes the whole row of k non-finite, i.e.
// zero; the block reproduces that with a row-wide flag (__syncthreads_or), so
// the rule holds whichever transforms run.
//
// Thread t of the CTA owns the points t, t + T, t + 2T, ... (T = full_threads:
// 256, 512 at N_t = 4096).  Shared
// memory holds three padded complex rows (the FFT ping-pong buffers) and three
// plain complex rows: the post-alpha field U, the RK accumulator and the stage
// field S, each read and written only by the thread owning the point.
#pragma once
#include "nl_impl.cuh"

// Shared memory of the full block: three padded complex row buffers (FFTs),
// the rows U, KS, S and the float row PH.  219,136 bytes at N_t = 4096.
template <int NT>
__host__ __device__ constexpr size_t full_smem_bytes() {
    return 3 * (size_t)fft_slots(NT) * sizeof(float2) + 3 * (size_t)NT * sizeof(float2) + (size_t)NT * sizeof(float);
}

struct FullRows {
    float2 *B0, *B1, *B2;  // padded FFT buffers
    float2 *U, *KS, *S;    // post-alpha field, RK accumulator, stage field (index t)
    float *PH;             // the stage's photo-ionisation term per point (index t)
};

template <int NT>
__device__ __forceinline__ FullRows full_rows(float2 *smem) {
    FullRows r;
    r.B0 = smem;
    r.B1 = smem + fft_slots(NT);
    r.B2 = smem + 2 * fft_slots(NT);
    r.U = smem + 3 * fft_slots(NT);
    r.KS = r.U + NT;
    r.S = r.KS + NT;
    r.PH = reinterpret_cast<float *>(r.S + NT);
    return r;
}

// photo (before alpha) as split() computes it: NaN for a NaN intensity or a
// NaN density (the reference's clip propagates NaN), 0 for +Inf intensity.
__device__ __forceinline__ float photo_term(float a2, float rho, const NLParams &p,
                                            const float4 *__restrict__ tab) {
    if (!p.photo_on) return 0.0f;
    const float I = a2 * p.invE2;
    if (isfinite(I)) {
        if (I < p.I_skip) return isnan(rho) ? rho : 0.0f;
        const float dep = isnan(rho) ? rho : fminf(fmaxf((p.rho_max - rho) * p.inv_rho_max, 0.0f), 1.0f);
        return photo_rate(I, p, tab) * dep;
    }
    return isnan(I) ? I : 0.0f;
}

// alpha = max(nan_to_num(photo + pp_abs rho), 0)
__device__ __forceinline__ float alpha_from(float photo, float rho, const NLParams &p) {
    const float ar = fmaf(p.pp_abs, rho, photo);
    return isfinite(ar) ? fmaxf(ar, 0.0f) : 0.0f;
}

__device__ __forceinline__ bool c_finite(float2 v) { return isfinite(v.x) && isfinite(v.y); }

// Threads of a full-physics CTA: 256, and 512 at N_t = 4096, where the row's
// buffers leave room for one CTA per SM and 512 threads give every radix-8 pass
// exactly one butterfly a thread (16 warps instead of 8 to hide the latency).
template <int NT>
__host__ __device__ constexpr int full_threads() {
    return NT >= 4096 ? 512 : NLSE_ROW_THREADS;
}

// Complex affine map x -> a x + b, and its composition (f first, then g).
struct CAff {
    float2 a, b;
};

__device__ __forceinline__ CAff caff_then(const CAff &f, const CAff &g) {
    return CAff{c_mul(g.a, f.a), c_add(c_mul(g.a, f.b), g.b)};
}

// Block-wide exclusive scan of one complex affine map per thread (thread
// order) and the composition of all of them; TT threads, wsum = 32 maps of
// shared scratch.  All threads call it.
template <int TT>
__device__ __forceinline__ void block_scan_caff(const CAff &v, CAff *wsum, CAff *pre, CAff *tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int NW = TT / 32;
    const CAff id{make_float2(1.0f, 0.0f), make_float2(0.0f, 0.0f)};
    CAff inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        CAff o;
        o.a.x = __shfl_up_sync(0xffffffffu, inc.a.x, off);
        o.a.y = __shfl_up_sync(0xffffffffu, inc.a.y, off);
        o.b.x = __shfl_up_sync(0xffffffffu, inc.b.x, off);
        o.b.y = __shfl_up_sync(0xffffffffu, inc.b.y, off);
        if (lane >= off) inc = caff_then(o, inc);
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        CAff w = lane < NW ? wsum[lane] : id;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            CAff o;
            o.a.x = __shfl_up_sync(0xffffffffu, w.a.x, off);
            o.a.y = __shfl_up_sync(0xffffffffu, w.a.y, off);
            o.b.x = __shfl_up_sync(0xffffffffu, w.b.x, off);
            o.b.y = __shfl_up_sync(0xffffffffu, w.b.y, off);
            if (lane >= off) w = caff_then(o, w);
        }
        if (lane < NW) wsum[lane] = w;
    }
    __syncthreads();
    CAff lex;
    lex.a.x = __shfl_up_sync(0xffffffffu, inc.a.x, 1);
    lex.a.y = __shfl_up_sync(0xffffffffu, inc.a.y, 1);
    lex.b.x = __shfl_up_sync(0xffffffffu, inc.b.x, 1);
    lex.b.y = __shfl_up_sync(0xffffffffu, inc.b.y, 1);
    if (lane == 0) lex = id;
    *pre = wid > 0 ? caff_then(wsum[wid - 1], lex) : lex;
    *tot = wsum[NW - 1];
    __syncthreads();  // wsum is free again
}

// The Raman convolution kerr_I's second term needs, Re F^-1[F[|S|^2] R_f], as
// the periodic solution of G[n] = z (G[n - 1] + I[n - 1]) (FullTabs::rz), with
// I = |S|^2: each thread composes the step maps of its chunk of C points, a
// block scan composes the chunks, G[-1] = G[N - 1] closes the period
// (G[-1] = b / (1 - a) for the whole row's map a x + b), and each thread walks
// its chunk again writing ramp Im G[n] -- times NT, as the FFT path leaves it
// unnormalised -- to Q[pidx(n)].  O(N) work instead of two row FFTs; the same
// circular convolution to ~1e-10 in exact arithmetic (raman_fit).
template <int NT, int TT>
__device__ __forceinline__ void raman_recurrence(const float2 *S, float2 *Q, float2 z, float ramp) {
    constexpr int C = NT >= TT ? NT / TT : 1;
    __shared__ CAff wsum[32];
    const int n0 = (int)threadIdx.x * C;
    CAff m{make_float2(1.0f, 0.0f), make_float2(0.0f, 0.0f)};
    __syncthreads();  // the chunks read points of S other threads wrote
    if (n0 < NT) {
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const float2 sp = S[(n0 + j - 1 + NT) & (NT - 1)];
            const float ip = fmaf(sp.x, sp.x, sp.y * sp.y);
            m = CAff{c_mul(z, m.a), c_mul(z, make_float2(m.b.x + ip, m.b.y))};
        }
    }
    CAff pre, tot;
    block_scan_caff<TT>(m, wsum, &pre, &tot);
    if (n0 < NT) {
        // G[-1] = tot.b / (1 - tot.a)
        const float2 d = make_float2(1.0f - tot.a.x, -tot.a.y);
        const float dd = fmaf(d.x, d.x, d.y * d.y);
        const float2 g0 = make_float2(fmaf(tot.b.x, d.x, tot.b.y * d.y) / dd, fmaf(tot.b.y, d.x, -tot.b.x * d.y) / dd);
        float2 G = c_add(c_mul(pre.a, g0), pre.b);  // G[n0 - 1]
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const float2 sp = S[(n0 + j - 1 + NT) & (NT - 1)];
            const float ip = fmaf(sp.x, sp.x, sp.y * sp.y);
            G = c_mul(z, make_float2(G.x + ip, G.y));
            Q[pidx(n0 + j)] = make_float2(ramp * G.y * (float)NT, 0.0f);
        }
    }
    __syncthreads();
}

// CTAs per SM the full-physics kernels are compiled for: what their shared
// memory admits, at most 2 (two CTAs of 256 threads, or one of 512 at N_t =
// 4096: <= 128 registers a thread either way; with the whole block inlined
// ptxas otherwise spends ~180).
template <int NT>
__host__ __device__ constexpr int full_min_blocks() {
    return (228 * 1024) / (int)(full_smem_bytes<NT>() + 1024) >= 2 ? 2 : 1;
}

// The transforms of split() itself (the Raman convolution, F[X] and the
// inverse of the filtered sum) take plain twiddle products: they produce k,
// which reaches the field only as dz k, so the fixed rounding of the twiddle
// table is scaled by the nonlinear phase of a step (<= ~0.05 rad) before it
// can repeat from step to step -- below 1e-5 of the field over 2000 z-steps.
// The row kernel's own transforms of the field keep the compensated products.
//
// k = split(S) for every point of the stage field S (shared, index t), left in
// a free FFT buffer (padded index) whose pointer is returned; synced, and the
// other buffers are free again.  All threads of the CTA call it.  Each thread
// evaluates photo-ionisation once per point (kept in m.PH for the second
// pass).  Out of line: the RK block calls it four times, and four inlined
// copies overflow the registers (one CTA per SM).
template <int NT>
__device__ __noinline__ float2 *rhs_full(const FullRows m, const float *__restrict__ rho,
                                         const float *__restrict__ rhos, const NLParams &p,
                                         const float4 *__restrict__ tab, const FullTabs &ft,
                                         const float2 *__restrict__ tw) {
    constexpr int TT = full_threads<NT>();
    constexpr int PP = (NT + TT - 1) / TT;  // points per thread
    constexpr float inv_n = 1.0f / (float)NT;
    const bool fft_path = ft.T != nullptr || ft.invU != nullptr;
    float2 *B0 = m.B0, *B1 = m.B1, *B2 = m.B2;
    const float2 *S = m.S;
    // Raman: kerr_I's convolution term Re F^-1[F[|S|^2] R_f], left in Q
    const float2 *Q = nullptr;
    if (ft.Rf && ft.riir) {
        raman_recurrence<NT, TT>(S, B0, ft.rz, ft.ramp);
        Q = B0;
    } else if (ft.Rf) {
        for (int t = threadIdx.x; t < NT; t += TT) {
            const float2 v = S[t];
            B0[pidx(t)] = make_float2(fmaf(v.x, v.x, v.y * v.y), 0.0f);
        }
        __syncthreads();
        float2 *R = fft_row<NT, false, TT, false>(B0, B1, tw);
        for (int f = threadIdx.x; f < NT; f += TT) R[pidx(f)] = c_mul(R[pidx(f)], __ldg(&ft.Rf[f]));
        __syncthreads();
        Q = fft_row<NT, true, TT, false>(R, R == B0 ? B1 : B0, tw);
    }
    // the pointwise terms; X1 (and X2) into the transform buffers on the FFT
    // path (a point's Q value is read before the same thread overwrites it)
    int bad = 0, any_x2 = 0, any_x3 = 0;
#pragma unroll
    for (int q = 0; q < PP; ++q) {
        const int t = (int)threadIdx.x + q * TT;
        if (NT % TT == 0 || t < NT) {
            const float2 s = S[t];
            const float a2 = fmaf(s.x, s.x, s.y * s.y);
            const float r = __ldg(&rho[t]), rs = rhos ? __ldg(&rhos[t]) : 0.0f;
            const float ph = photo_term(a2, r, p, tab);
            any_x2 |= ph != 0.0f;
            any_x3 |= r != 0.0f || rs != 0.0f;
            m.PH[t] = ph;
            const float kr = Q ? Q[pidx(t)].x * inv_n : 0.0f;
            const float K = fmaf(p.kp, a2, p.kp_raman * kr);  // kerr_pref * kerr_I
            const float2 x1 = make_float2(-K * s.y, K * s.x);   // i K S
            const float2 x2 = c_scale(s, ph);
            const float2 x3 = c_mul(s, make_float2(-p.pp_abs * r, fmaf(p.ste_pref, rs, -p.pp_def * r)));
            bad |= !(c_finite(x1) && c_finite(x2) && c_finite(x3));
            if (ft.T) {
                B0[pidx(t)] = x1;
                B2[pidx(t)] = x2;
            } else if (ft.invU) {
                B0[pidx(t)] = c_add(c_sub(x1, x2), x3);
            }
        }
    }
    bad = __syncthreads_or(bad);  // also orders the buffer writes before the transforms
    // On the self-steepening path X2 and X3 have transforms of their own: a
    // row where the photo-ionisation term (X2) or the carrier densities (X3)
    // are zero at every point has an exactly zero transform of that term, and
    // it is left out (the results are the same but for the sign of zeros).
    if (ft.T) {
        any_x2 = __syncthreads_or(any_x2);
        any_x3 = __syncthreads_or(any_x3);
    }
    float2 *Y = nullptr;          // the spectral part of k (inverse-transformed, unnormalised)
    if (fft_path && !bad) {
        float2 *C;
        if (ft.T) {
            float2 *P1 = fft_row<NT, false, TT, false>(B0, B1, tw);
            float2 *fr = P1 == B0 ? B1 : B0;
            float2 *P2 = B2;   // F[X2], or (no X2 transform) the unused X2 buffer
            if (any_x2) P2 = fft_row<NT, false, TT, false>(B2, fr, tw);
            float2 *fr2 = P2 == B2 ? fr : B2;  // the buffer neither P1 nor P2 occupies
            for (int f = threadIdx.x; f < NT; f += TT) {
                const float T = __ldg(&ft.T[f]);
                const float2 a = P1[pidx(f)], b = any_x2 ? P2[pidx(f)] : make_float2(0.0f, 0.0f);
                // T^2 F[X1] - T F[X2] = T (T F[X1] - F[X2])
                P1[pidx(f)] = c_scale(make_float2(fmaf(T, a.x, -b.x), fmaf(T, a.y, -b.y)), T);
            }
            C = P1;
            if (ft.invU && !any_x3) {
                // F[X3] = 0: only the U^-1 factor
                for (int f = threadIdx.x; f < NT; f += TT) C[pidx(f)] = c_scale(C[pidx(f)], __ldg(&ft.invU[f]));
                __syncthreads();
                Y = fft_row<NT, true, TT, false>(C, P2, tw);
            } else if (ft.invU) {
                // F[X3] through the two free buffers, then the U^-1 factor
#pragma unroll
                for (int q = 0; q < PP; ++q) {
                    const int t = (int)threadIdx.x + q * TT;
                    if (NT % TT == 0 || t < NT) {
                        const float r = __ldg(&rho[t]), rs = rhos ? __ldg(&rhos[t]) : 0.0f;
                        P2[pidx(t)] = c_mul(S[t], make_float2(-p.pp_abs * r, fmaf(p.ste_pref, rs, -p.pp_def * r)));
                    }
                }
                __syncthreads();
                float2 *P3 = fft_row<NT, false, TT, false>(P2, fr2, tw);
                for (int f = threadIdx.x; f < NT; f += TT)
                    C[pidx(f)] = c_scale(c_add(C[pidx(f)], P3[pidx(f)]), __ldg(&ft.invU[f]));
                __syncthreads();
                Y = fft_row<NT, true, TT, false>(C, P3 == P2 ? fr2 : P2, tw);
            } else {
                __syncthreads();
                Y = fft_row<NT, true, TT, false>(C, P2, tw);
            }
        } else {
            C = fft_row<NT, false, TT, false>(B0, B1, tw);
            for (int f = threadIdx.x; f < NT; f += TT) C[pidx(f)] = c_scale(C[pidx(f)], __ldg(&ft.invU[f]));
            __syncthreads();
            Y = fft_row<NT, true, TT, false>(C, C == B0 ? B1 : B0, tw);
        }
    }
    // k per point, written where the thread read its Y (or Q) value: the same
    // point of a buffer nothing else reads any more
    float2 *K = Y ? Y : B0;
#pragma unroll
    for (int q = 0; q < PP; ++q) {
        const int t = (int)threadIdx.x + q * TT;
        if (NT % TT == 0 || t < NT) {
            const float2 s = S[t];
            const float a2 = fmaf(s.x, s.x, s.y * s.y);
            const float r = __ldg(&rho[t]), rs = rhos ? __ldg(&rhos[t]) : 0.0f, ph = m.PH[t];
            const float al = alpha_from(ph, r, p);
            float2 k;
            if (fft_path) {
                k = bad ? make_float2(0.0f, 0.0f) : c_scale(Y[pidx(t)], inv_n);
                if (!ft.invU)  // X3 pointwise
                    k = c_add(k, c_mul(s, make_float2(-p.pp_abs * r, fmaf(p.ste_pref, rs, -p.pp_def * r))));
                k = make_float2(fmaf(al, s.x, k.x), fmaf(al, s.y, k.y));
            } else {
                // X1 - X2 + X3 + alpha S = i w S + (alpha - photo - pp_abs rho) S
                const float kr = Q ? Q[pidx(t)].x * inv_n : 0.0f;
                const float w = fmaf(p.kp, a2, p.kp_raman * kr) + fmaf(p.ste_pref, rs, -p.pp_def * r);
                const float corr = al - fmaf(p.pp_abs, r, ph);
                k = make_float2(fmaf(corr, s.x, -w * s.y), fmaf(corr, s.y, w * s.x));
            }
            if (bad || !(a2 >= 1e-30f) || !c_finite(k)) k = make_float2(0.0f, 0.0f);
            K[pidx(t)] = k;
        }
    }
    __syncthreads();
    return K;
}

// alpha/2, RK4 on split(), alpha/2 (Integrator.step, integrator.py:140-147)
// for the row held in m.U (index t; all threads); rho / rho_s frozen.  On
// return (synced) m.U holds the new field.
template <int NT>
__device__ __forceinline__ void nl_block_full(const FullRows &m, const float *__restrict__ rho,
                                              const float *__restrict__ rhos, float dz, const NLParams &p,
                                              const float4 *__restrict__ tab, const FullTabs &ft,
                                              const float2 *__restrict__ tw) {
    constexpr int TT = full_threads<NT>();
    const float hdz = 0.5f * dz;
    float2 *U = m.U, *KS = m.KS, *S = m.S;
    for (int t = threadIdx.x; t < NT; t += TT) {
        const float2 u = U[t];
        const float r = __ldg(&rho[t]);
        const float al = alpha_from(photo_term(fmaf(u.x, u.x, u.y * u.y), r, p, tab), r, p);
        U[t] = S[t] = c_damp(u, -hdz * al);
    }
    // k1..k4; KS = k1 + 2 k2 + 2 k3 + k4 (each thread touches only its points)
    const float2 *K = rhs_full<NT>(m, rho, rhos, p, tab, ft, tw);
    for (int t = threadIdx.x; t < NT; t += TT) {
        const float2 k = K[pidx(t)];
        KS[t] = k;
        S[t] = make_float2(fmaf(hdz, k.x, U[t].x), fmaf(hdz, k.y, U[t].y));
    }
    __syncthreads();
    K = rhs_full<NT>(m, rho, rhos, p, tab, ft, tw);
    for (int t = threadIdx.x; t < NT; t += TT) {
        const float2 k = K[pidx(t)];
        KS[t] = make_float2(fmaf(2.0f, k.x, KS[t].x), fmaf(2.0f, k.y, KS[t].y));
        S[t] = make_float2(fmaf(hdz, k.x, U[t].x), fmaf(hdz, k.y, U[t].y));
    }
    __syncthreads();
    K = rhs_full<NT>(m, rho, rhos, p, tab, ft, tw);
    for (int t = threadIdx.x; t < NT; t += TT) {
        const float2 k = K[pidx(t)];
        KS[t] = make_float2(fmaf(2.0f, k.x, KS[t].x), fmaf(2.0f, k.y, KS[t].y));
        S[t] = make_float2(fmaf(dz, k.x, U[t].x), fmaf(dz, k.y, U[t].y));
    }
    __syncthreads();
    K = rhs_full<NT>(m, rho, rhos, p, tab, ft, tw);
    for (int t = threadIdx.x; t < NT; t += TT) KS[t] = c_add(KS[t], K[pidx(t)]);
    const float s6 = dz * (1.0f / 6.0f);
    for (int t = threadIdx.x; t < NT; t += TT) {
        float2 u = make_float2(fmaf(s6, KS[t].x, U[t].x), fmaf(s6, KS[t].y, U[t].y));
        const float r = __ldg(&rho[t]);
        const float al = alpha_from(photo_term(fmaf(u.x, u.x, u.y * u.y), r, p, tab), r, p);
        U[t] = c_damp(u, -hdz * al);
    }
    __syncthreads();
}
