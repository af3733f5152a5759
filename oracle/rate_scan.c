/*
 * FP64 C restatement of the reference's carrier-rate kernel.
 *
 * TEST INFRASTRUCTURE (the oracle): only tests, the smoke check and the CPU
 * baseline of bench.py load this library.  It is never on the product path.
 *
 * Follows deliverable (3)/sim/kernels.py:
 *   - rate lookup  : interpolate_pi_rate, kernels.py:14-26 (linear in log10 I
 *                    over a uniform table; sanitise I; clamp to [Imin, Imax];
 *                    clamp the index; non-finite/negative result -> 0)
 *   - exponential  : exact_exp_step, kernels.py:28-34
 *                    x' = e^{L dt} x + S dt phi1(L dt), phi1 by series for
 *                    |L dt| <= 1e-6; non-finite/negative -> 0
 *   - the march    : solve_rate_equation_kernel, kernels.py:36-106
 *                    trapezoid averages of I and W between t and t+1, the
 *                    depletion factor clamp(1 - ne/na, 0, 1), the optional
 *                    self-trapped-exciton population, and the ne+ns <= na
 *                    rescale.
 * Rows are independent (one GPU thread per radius in the reference); here an
 * OpenMP loop over rows.
 */
#include <math.h>
#include <stddef.h>

static double rate_lookup(double I, const double *table, int n, double log_min,
                          double inv_step, double Imin, double Imax)
{
    if (!isfinite(I) || I < 0.0) I = 0.0;
    if (I < Imin) I = Imin;
    if (I > Imax) I = Imax;
    double pos = (log10(I) - log_min) * inv_step;
    int k = (int)pos;
    if (k < 0) k = 0;
    if (k > n - 2) k = n - 2;
    double w = table[k] + (pos - (double)k) * (table[k + 1] - table[k]);
    if (!isfinite(w) || w < 0.0) return 0.0;
    return w;
}

static double exp_step(double x, double S, double L, double dt)
{
    double z = L * dt;
    double p;
    if (fabs(z) > 1e-6)
        p = (exp(z) - 1.0) / z;
    else
        p = 1.0 + z * (0.5 + z * (1.0 / 6.0 + z / 24.0));
    double y = exp(z) * x + S * dt * p;
    if (!isfinite(y) || y < 0.0) return 0.0;
    return y;
}

void oracle_rate_scan(const double *E /* interleaved re,im; Nr x Nt */,
                      double *ne, double *ns, int Nr, int Nt, double dt,
                      double field_to_I, double beta_g, double beta_s, double na,
                      double inv_tau_r, double inv_tau_ste, int enable_ste,
                      const double *lut, const double *lut_s, int lut_n,
                      double log_min, double inv_step, double Imin, double Imax)
{
    int r;
#pragma omp parallel for schedule(static)
    for (r = 0; r < Nr; ++r) {
        size_t row = (size_t)r * (size_t)Nt;
        double xe = ne[row], xs = ns[row];
        if (!isfinite(xe) || xe < 0.0) xe = 0.0;
        if (!isfinite(xs) || xs < 0.0) xs = 0.0;
        const double *e0 = E + 2 * row;
        double Ic = (e0[0] * e0[0] + e0[1] * e0[1]) * field_to_I;
        double Wc = rate_lookup(Ic, lut, lut_n, log_min, inv_step, Imin, Imax);
        double Wsc = enable_ste ? rate_lookup(Ic, lut_s, lut_n, log_min, inv_step, Imin, Imax) : 0.0;
        for (int t = 0; t + 1 < Nt; ++t) {
            const double *e1 = E + 2 * (row + t + 1);
            double In = (e1[0] * e1[0] + e1[1] * e1[1]) * field_to_I;
            double Wn = rate_lookup(In, lut, lut_n, log_min, inv_step, Imin, Imax);
            double Wsn = enable_ste ? rate_lookup(In, lut_s, lut_n, log_min, inv_step, Imin, Imax) : 0.0;
            double Ia = 0.5 * (Ic + In), Wa = 0.5 * (Wc + Wn), Wsa = 0.5 * (Wsc + Wsn);
            double dep = 1.0 - xe / na;
            if (dep < 0.0) dep = 0.0;
            if (dep > 1.0) dep = 1.0;
            double reion = enable_ste ? (Wsa + beta_s * Ia * xe) : 0.0;
            double Se = Wa * dep + (enable_ste ? reion * (xs / na) : 0.0);
            double Le = beta_g * Ia * dep - inv_tau_r;
            double Ss = enable_ste ? inv_tau_r * xe : 0.0;
            double Ls = enable_ste ? -reion / na - inv_tau_ste : 0.0;
            double ye = exp_step(xe, Se, Le, dt);
            double ys = enable_ste ? exp_step(xs, Ss, Ls, dt) : 0.0;
            if (ye + ys > na) {
                double k = na / (ye + ys);
                ye *= k;
                ys *= k;
            }
            ne[row + t + 1] = ye;
            ns[row + t + 1] = ys;
            xe = ye;
            xs = ys;
            Ic = In;
            Wc = Wn;
            Wsc = Wsn;
        }
    }
}
