// Runtime dispatch of the fused row kernels over N_t (the kernels and their
// per-N_t launchers are in k_rowfused.cuh, instantiated in k_row_n*.cu), and
// the small helper kernels of the split forms.
#include <math.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "k_rowfused.cuh"

cudaError_t launch_row_entry(const RowFusedArgs &a, const float2 *u, float *F32, __nv_bfloat16 *Fb, float *rho,
                             int do_scan, cudaStream_t st) {
    NLSE_DISPATCH_NT(a.logNt, return RowKernels<NT>::entry(a, u, F32, Fb, rho, do_scan, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_nl_full(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D,
                               const float *rho, int g, cudaStream_t st) {
    NLSE_DISPATCH_NT_FULL(a.logNt, return RowKernels<NT>::nl_full(a, F32, Fb, D, rho, g, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_nl(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, const float *rho,
                          int g, int plan, cudaStream_t st) {
    NLSE_DISPATCH_NT(a.logNt, return RowKernels<NT>::nl(a, F32, Fb, D, rho, g, plan, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_next(const RowFusedArgs &a, float *F32, __nv_bfloat16 *Fb, const float *D, float *rho,
                            float2 *u_out, int write_state, int do_scan, int apply_mask, int g, int plan,
                            cudaStream_t st) {
    NLSE_DISPATCH_NT(a.logNt, return RowKernels<NT>::next(a, F32, Fb, D, rho, u_out, write_state, do_scan,
                                                          apply_mask, g, plan, st));
    return cudaErrorInvalidValue;
}

cudaError_t launch_row_batch(int kind, int logNt, const PulseTable &T, const BatchCall *calls, const int2 *work,
                             int nblocks, int flag, int g, int plan, cudaStream_t st) {
    if (kind == 3) {
        NLSE_DISPATCH_NT_FULL(logNt, return RowKernels<NT>::batch(kind, T, calls, work, nblocks, flag, g, plan, st));
    } else {
        NLSE_DISPATCH_NT(logNt, return RowKernels<NT>::batch(kind, T, calls, work, nblocks, flag, g, plan, st));
    }
    return cudaErrorInvalidValue;
}

// Split-FP16 form: before the entry kernel writes GEMM input 0 = F[u], its
// "previous maximum" is the bound Nt max |u| >= max |F[u]| (slot 2), and the
// slot input 0 fills is cleared.
__global__ void k_field_bound(const float2 *__restrict__ u, size_t n, int Nt, int *__restrict__ scale) {
    float mx = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = u[i];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    mx = block_max(mx);
    if (threadIdx.x == 0) atomicMax(&scale[NLSE_SC_MAX + 2], __float_as_int(mx * (float)Nt * 1.5f));
}

cudaError_t launch_field_bound(const float2 *u, size_t n, int Nt, int *scale, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(scale + NLSE_SC_MAX, 0, 3 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    k_field_bound<<<2 * 152, NLSE_ROW_THREADS, 0, st>>>(u, n, Nt, scale);
    return cudaGetLastError();
}

// FP32 planar field -> BF16 hi/lo terms (diagnostic path of nlse_debug_operator_product).
__global__ void k_split_field(const float *__restrict__ w, __nv_bfloat16 *__restrict__ hi, size_t lo_off,
                              size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = w[i];
        __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        hi[lo_off + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

cudaError_t launch_split_field(const float *w, __nv_bfloat16 *hi, size_t lo_off, size_t n, cudaStream_t st) {
    k_split_field<<<1024, 256, 0, st>>>(w, hi, lo_off, n);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ row plans (autotuner)
// Per device and N_t, the fastest of the plans of row_nl and of row_next
// (k_rowfused.cuh: the same arithmetic, so the pick never changes results).
// Stored as pick + 1 (0 = not tuned yet); set_row_plan pins a pick and bumps
// the generation, which the batches' captured graphs are keyed on.
#define NLSE_PLAN_DEVICES 64
static std::atomic<int> g_row_plan[NLSE_PLAN_DEVICES][14][2];
static std::atomic<int> g_row_plan_gen{0};
static std::mutex g_row_plan_mu;

static int plan_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NLSE_PLAN_DEVICES) return -1;
    return dev;
}

int row_plan(int logNt, int kind) {
    const int dev = plan_device();
    if (dev < 0 || logNt < 0 || logNt > 13) return 0;
    const int v = g_row_plan[dev][logNt][kind].load(std::memory_order_relaxed);
    return v > 0 ? v - 1 : 0;
}

int row_plan_generation() { return g_row_plan_gen.load(std::memory_order_relaxed); }

int row_plan_get(int logNt, int kind) {
    const int dev = plan_device();
    if (dev < 0 || logNt < 0 || logNt > 13) return -1;
    return g_row_plan[dev][logNt][kind].load(std::memory_order_relaxed) - 1;
}

int row_plan_set(int logNt, int kind, int plan) {
    const int dev = plan_device();
    if (dev < 0 || logNt < 0 || logNt > 13 || plan < -1 || plan > (kind == 0 ? 2 : 1)) return -1;
    g_row_plan[dev][logNt][kind].store(plan + 1, std::memory_order_relaxed);
    g_row_plan_gen.fetch_add(1, std::memory_order_relaxed);
    return 0;
}

// Tuning rows: a constant spectrum bin (a flat row of intensity 1e11 W/cm^2
// after the inverse transform) in every row's Re plane, zero product and
// densities; the nonlinear block and the march then run their full paths.
__global__ void k_tune_fill(float *__restrict__ F32, int rows, int NT, float c) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) F32[(size_t)r * NT] = c;
}

namespace {
// plans of a kind that exist for N_t (row_nl: 0, 2 and from 512 on 1; row_next: 0, and from 2048 on 1)
template <int NT>
int plan_mask(int kind) {
    return kind == 0 ? (1 | 4 | (nl_plan1_ok<NT>() ? 2 : 0)) : (1 | (next_plan1_ok<NT>() ? 2 : 0));
}
}  // namespace

cudaError_t row_plan_tune(int logNt, int Nr, const float2 *tw, const float *lut, const float4 *pchip,
                          const float *mask_r, const NLParams &nl, const ScanParams &sc, float2 *Pt_scratch,
                          int *scale) {
    const int dev = plan_device();
    if (dev < 0 || logNt < 4 || logNt > 13) return cudaSuccess;
    std::lock_guard<std::mutex> lock(g_row_plan_mu);
    const int NT = 1 << logNt;
    int want[2], mask[2];
    for (int kind = 0; kind < 2; ++kind) {
        int m = 1;
        NLSE_DISPATCH_NT(logNt, m = plan_mask<NT>(kind));
        mask[kind] = m;
        want[kind] = m != 1 && g_row_plan[dev][logNt][kind].load() == 0;
        if (m == 1 && g_row_plan[dev][logNt][kind].load() == 0) g_row_plan[dev][logNt][kind].store(1);
    }
    if (!want[0] && !want[1]) return cudaSuccess;
    // enough rows to fill the GPU a few times over, within the context's radial size
    int R = (2 << 20) / NT;
    R = R < 64 ? 64 : (R > 1024 ? 1024 : R);
    R = R < Nr ? R : Nr;
    float *F32 = nullptr, *D = nullptr, *rho = nullptr;
    __nv_bfloat16 *Fb = nullptr;
    int *stats = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const size_t pts = (size_t)R * NT;
    cudaError_t e = cudaMalloc((void **)&F32, 2 * pts * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&D, 2 * pts * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&rho, pts * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&Fb, 4 * pts * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&stats, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(F32, 0, 2 * pts * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(D, 0, 2 * pts * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(rho, 0, pts * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(stats, 0, 4 * sizeof(int));
    if (e == cudaSuccess) {
        std::vector<float2> pt(2 * (size_t)NT, make_float2(0.0f, 0.0f));
        for (int k = 0; k < NT; ++k) pt[k] = make_float2(1.0f, 0.0f);
        e = cudaMemcpy(Pt_scratch, pt.data(), pt.size() * sizeof(float2), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        k_tune_fill<<<(R + 255) / 256, 256>>>(F32, R, NT, (float)((double)NT * sqrt(1e11 / (double)nl.invE2)));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    RowFusedArgs a{};
    a.Nr = R;
    a.Nt = NT;
    a.logNt = logNt;
    a.Nrp = R;
    a.tw = tw;
    a.Pt = Pt_scratch;
    a.mask_r = mask_r;
    a.lut = lut;
    a.pchip = pchip;
    a.nl = nl;
    a.sc = sc;
    a.sc.ste = 0;
    a.dz = 2.5e-6f;
    a.stats = stats;
    a.rho_s = nullptr;
    a.ft = FullTabs{nullptr, nullptr, nullptr, make_float2(0.0f, 0.0f), 0.0f, 0};
    a.f16 = 0;
    a.scale = scale;
    // Every plan runs once untimed (module load, instruction cache, the clock
    // leaving idle), then the plans are timed in turn over several rounds and
    // each keeps its fastest round: a plan timed while the clock still ramps
    // up, or in a disturbed round, is not chosen for that.
    auto run = [&](int kind, int plan) {
        return kind == 0 ? launch_row_nl(a, F32, Fb, D, rho, 0, plan, 0)
                         : launch_row_next(a, F32, Fb, D, rho, nullptr, 1, 1, 1, 1, plan, 0);
    };
    for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
        if (!want[kind]) continue;
        float best[3] = {1e30f, 1e30f, 1e30f};
        for (int plan = 0; plan < 3 && e == cudaSuccess; ++plan)
            if (mask[kind] & (1 << plan)) e = run(kind, plan);
        for (int round = 0; round < 3 && e == cudaSuccess; ++round) {
            for (int plan = 0; plan < 3 && e == cudaSuccess; ++plan) {
                if (!(mask[kind] & (1 << plan))) continue;
                e = cudaEventRecord(e0, 0);
                for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) e = run(kind, plan);
                if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 1e30f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e == cudaSuccess && ms < best[plan]) best[plan] = ms;
            }
        }
        int pick = 0;
        for (int plan = 1; plan < 3; ++plan)
            if (best[plan] < best[pick]) pick = plan;
        if (e == cudaSuccess) g_row_plan[dev][logNt][kind].store(pick + 1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(F32);
    cudaFree(D);
    cudaFree(rho);
    cudaFree(Fb);
    cudaFree(stats);
    return e;
}
