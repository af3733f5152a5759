// Allocation-free half-linear step for callers that cannot call cudaMalloc.
//
// Some callers run where device allocation is not available to them: a host
// application that owns every device buffer through its own memory pool and
// forbids allocations from plugins, a real-time loop that must not hit the
// driver's allocator, or code that runs before the caller can create a
// context.  nlse_half_linear_noalloc serves them: it takes every table and the
// field as caller-owned device pointers, needs no nlse_ctx, and keeps its
// intermediate field and twiddle table in the file-scope array below.
//
// The array is a fixed 4 MiB + 201 KiB of device memory that every GPU which
// loads this library holds until the process exits.  Its address is looked up
// once per device (cudaGetSymbolAddress, with that device current) on the
// first call made on that device; make that first call before any stream
// capture.  Every call shares the one array and it keeps the last call's
// contents (each call rewrites all of it that it reads), so calls that
// overlap on the GPU -- on two streams, or from two threads -- race.
#include <math.h>
#include <stdarg.h>

#include <mutex>

#include "nlse_internal.cuh"

#define NLSE_NOALLOC_MAX_POINTS (1 << 19)  // Nr * Nt complex64 points: 4 MiB

static __device__ __align__(256) float2 g_noalloc_scratch[NLSE_NOALLOC_MAX_POINTS + 2 * fft_tw_size(NLSE_MAX_NT)];

static float2 *g_scratch_ptr[64];
static std::mutex g_scratch_mu;

// Device address of the scratch array on the current device (set-up on first use).
static cudaError_t scratch_for_current_device(float2 **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = (float2 *)p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// The row FFT's twiddle table (per-pass row layout), FP64 then rounded: the
// same values as a context's table.
__global__ void k_noalloc_twiddles(float2 *__restrict__ tw, int Nt) {
    const int n = fft_tw_size(Nt);
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) {
        int m;
        fft_tw_entry(Nt, e, &m);
        double s = 0.0, c = 0.0;
        if (m >= 0) sincospi(-2.0 * (double)m / (double)Nt, &s, &c);
        const float2 h = make_float2((float)c, (float)s);
        tw[e] = h;
        tw[n + e] = make_float2((float)(c - (double)h.x), (float)(s - (double)h.y));
    }
}

static int fail(int status, const char *fmt, ...);

extern "C" int nlse_half_linear_noalloc(const float *Y, const void *Pt, const void *Pr, void *u, int Nr, int Nt,
                                        void *stream) {
    if (!Y || !Pt || !Pr || !u) return fail(NLSE_ERR_INVALID_ARG, "a pointer argument is NULL");
    if (Nr < 1 || Nt < 16 || Nt > NLSE_MAX_NT || (Nt & (Nt - 1)))
        return fail(NLSE_ERR_INVALID_ARG, "Nr=%d, Nt=%d: Nt must be a power of two in [16, %d]", Nr, Nt,
                    NLSE_MAX_NT);
    if ((size_t)Nr * (size_t)Nt > NLSE_NOALLOC_MAX_POINTS)
        return fail(NLSE_ERR_INVALID_ARG,
                    "Nr*Nt = %zu exceeds the %d points of the static scratch of nlse_half_linear_noalloc",
                    (size_t)Nr * (size_t)Nt, NLSE_NOALLOC_MAX_POINTS);
    if ((uintptr_t)u % 16) return fail(NLSE_ERR_INVALID_ARG, "u is not 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    float2 *scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) return fail(NLSE_ERR_CUDA, "scratch set-up: %s", cudaGetErrorString(e));
    float2 *work = scratch, *tw = scratch + NLSE_NOALLOC_MAX_POINTS;
    int logNt = 0;
    while ((1 << logNt) < Nt) ++logNt;

    k_noalloc_twiddles<<<(fft_tw_size(Nt) + 255) / 256, 256, 0, st>>>(tw, Nt);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_gemm_f32(Y, (const float *)u, (float *)work, Nr, 2 * Nt, Nr, nullptr, st);
    if (e == cudaSuccess)
        e = launch_fft_phase_ifft_tables(work, Nr, Nt, logNt, tw, (const float2 *)Pt, (const float2 *)Pr, st);
    if (e == cudaSuccess) e = launch_gemm_f32(Y, (const float *)work, (float *)u, Nr, 2 * Nt, Nr, nullptr, st);
    if (e != cudaSuccess) return fail(NLSE_ERR_CUDA, "nlse_half_linear_noalloc: %s", cudaGetErrorString(e));
    return NLSE_OK;
}

static int fail(int status, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    nlse_set_thread_error(status, buf);
    return status;
}
