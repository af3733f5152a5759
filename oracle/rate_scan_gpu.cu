// FP64 GPU restatement of the reference's carrier-rate kernel -- the same
// arithmetic as oracle/rate_scan.c (kernels.py:14-106), one thread per radius.
//
// TEST INFRASTRUCTURE (the oracle): used only by the tests' FP64 GPU
// reference for long (1 cm) runs; never on the product path.
#include <cuda_runtime.h>
#include <math.h>

__device__ static double rate_lookup(double I, const double *table, int n, double log_min, double inv_step,
                                     double Imin, double Imax) {
    if (!isfinite(I) || I < 0.0) I = 0.0;
    if (I < Imin) I = Imin;
    if (I > Imax) I = Imax;
    double pos = (log10(I) - log_min) * inv_step;
    int k = (int)pos;
    if (k < 0) k = 0;
    if (k > n - 2) k = n - 2;
    double w = table[k] + (pos - (double)k) * (table[k + 1] - table[k]);
    return (!isfinite(w) || w < 0.0) ? 0.0 : w;
}

__device__ static double exp_step(double x, double S, double L, double dt) {
    double z = L * dt;
    double p = fabs(z) > 1e-6 ? (exp(z) - 1.0) / z : 1.0 + z * (0.5 + z * (1.0 / 6.0 + z / 24.0));
    double y = exp(z) * x + S * dt * p;
    return (!isfinite(y) || y < 0.0) ? 0.0 : y;
}

__global__ void k_oracle_scan(const double2 *E, double *ne, int Nr, int Nt, double dt, double f2I, double beta,
                              double na, double itr, const double *lut, int lut_n, double lmin, double idl,
                              double Imin, double Imax) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= Nr) return;
    size_t row = (size_t)r * Nt;
    double x = 0.0;
    ne[row] = 0.0;
    double2 e0 = E[row];
    double Ic = (e0.x * e0.x + e0.y * e0.y) * f2I;
    double Wc = rate_lookup(Ic, lut, lut_n, lmin, idl, Imin, Imax);
    for (int t = 0; t + 1 < Nt; ++t) {
        double2 e1 = E[row + t + 1];
        double In = (e1.x * e1.x + e1.y * e1.y) * f2I;
        double Wn = rate_lookup(In, lut, lut_n, lmin, idl, Imin, Imax);
        double Ia = 0.5 * (Ic + In), Wa = 0.5 * (Wc + Wn);
        double dep = 1.0 - x / na;
        if (dep < 0.0) dep = 0.0;
        if (dep > 1.0) dep = 1.0;
        double y = exp_step(x, Wa * dep, beta * Ia * dep - itr, dt);
        if (y > na) y *= na / y;
        ne[row + t + 1] = y;
        x = y;
        Ic = In;
        Wc = Wn;
    }
}

extern "C" int oracle_rate_scan_gpu(const void *E, double *ne, int Nr, int Nt, double dt, double f2I, double beta,
                                    double na, double itr, const double *lut, int lut_n, double lmin, double idl,
                                    double Imin, double Imax, void *stream) {
    k_oracle_scan<<<(Nr + 127) / 128, 128, 0, (cudaStream_t)stream>>>((const double2 *)E, ne, Nr, Nt, dt, f2I, beta,
                                                                     na, itr, lut, lut_n, lmin, idl, Imin, Imax);
    return (int)cudaGetLastError();
}
