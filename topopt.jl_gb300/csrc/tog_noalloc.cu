// Allocation-free variant of the OC update (tog_oc_update_noalloc).
//
// Some callers cannot call cudaMalloc: a host framework that owns and
// pre-partitions all device memory, a memory-capped service, or a caller whose
// optimisation loop must not allocate between iterations.  This entry point
// runs the optimality-criteria bisection of tog_oc_update on device arrays the
// caller passes in, and keeps its only scratch -- the per-element OC factors,
// the block partial sums and the bisection state -- in one static __device__
// array of this file.  It has no handle, so every cell is free: the fixed
// (black / white) cells of tog_set_fixed_elements are not held here.
//
// Limits and rules of use:
//   * at most kNoallocMaxCells cells (8 MiB of factors); larger n is rejected.
//   * every GPU that loads the library holds the array (about 8.1 MiB) until
//     the process exits.
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, that device current); make that
//     first call before any stream capture.  The address is kept for the
//     process: a cudaDeviceReset between calls would leave it stale.
//   * the 100 bisection launches are always issued (no host synchronisation);
//     the ones after convergence return at once.
//   * all calls share the array and it keeps the last call's contents; each
//     call re-initialises the bisection state and counters it relies on.
//     Calls that overlap on the GPU (different streams, or threads) race on it.
//   * no cudaMalloc, cudaFree or allocating library routine is called.
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/topopt_gb300.h"
#include "tog_internal.h"
#include "tog_reduce.cuh"

namespace {

constexpr long long kNoallocMaxCells = 1LL << 20;   // 1,048,576 cells
constexpr int kNoallocBlocks = 1024;                // grid size of every launch
constexpr int kNoallocThreads = 256;
constexpr int kNoallocMaxSteps = 100;

struct NoallocScratch {
    tog::OcState oc;
    double partials[4 * kNoallocBlocks];
    double B[kNoallocMaxCells];
};

// The scratch.  In host code `g_noalloc_scratch` names a host-side stand-in, not
// device memory: kernels receive the address looked up by noalloc_scratch().
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
NoallocScratch* g_noalloc_ptr[kMaxDevices] = {};

int noalloc_fail(int code, const std::string& msg) { return tog::set_error(code, msg.c_str()); }

// Device address of the scratch on the current device (looked up once per device).
int noalloc_scratch(NoallocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(TOG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(TOG_ERR_ARG, "device ordinal beyond 64");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return noalloc_fail(TOG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<NoallocScratch*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return TOG_OK;
}

__global__ void __launch_bounds__(kNoallocThreads) k_na_prep(const double* __restrict__ x,
                                                             const double* __restrict__ dc,
                                                             const double* __restrict__ dv, long long n,
                                                             double volfrac, double move, NoallocScratch* S) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        S->B[e] = x[e] * sqrt(fmax(0.0, -dc[e]) / dv[e]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        tog::OcState& oc = S->oc;
        oc.l1 = 0.0;
        oc.l2 = 1e9;
        oc.tol = 1e-3;
        oc.target = volfrac;
        oc.move = move;
        oc.vol = 0.0;
        oc.change = 0.0;
        oc.lmid = 0.0;
        oc.steps = 0;
        oc.done = 0;
        oc.maxsteps = kNoallocMaxSteps;
        for (int i = 0; i < 4; ++i) oc.cnt[i] = 0u;   // last-block counters must start at zero
    }
}

__global__ void __launch_bounds__(kNoallocThreads) k_na_step(const double* __restrict__ x,
                                                             const double* __restrict__ w, long long n,
                                                             NoallocScratch* S) {
    tog::OcState& oc = S->oc;
    if (oc.done) return;
    const double lmid = 0.5 * (oc.l2 + oc.l1);
    const double s = 1.0 / sqrt(lmid);
    const double move = oc.move;
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double xe = x[e];
        const double xn = fmin(fmin(1.0, xe + move), fmax(fmax(0.0, xe - move), S->B[e] * s));
        acc = fma(w[e], xn, acc);
    }
    double v[1] = {acc}, tot[1];
    if (tog::grid_reduce_last<1>(v, S->partials, &oc.cnt[0], tot)) {
        if (threadIdx.x == 0) {
            oc.vol = tot[0];
            if (tot[0] > oc.target)
                oc.l1 = lmid;
            else
                oc.l2 = lmid;
            oc.steps += 1;
            if ((oc.l2 - oc.l1) / (oc.l1 + oc.l2) <= oc.tol || oc.steps >= oc.maxsteps) oc.done = 1;
        }
    }
}

__global__ void __launch_bounds__(kNoallocThreads) k_na_final(const double* __restrict__ x,
                                                              const double* __restrict__ w,
                                                              double* __restrict__ xnew, long long n,
                                                              NoallocScratch* S, double* __restrict__ result) {
    tog::OcState& oc = S->oc;
    const double lmid = 0.5 * (oc.l2 + oc.l1);
    const double s = 1.0 / sqrt(lmid);
    const double move = oc.move;
    double mx = 0.0, vol = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double xe = x[e];
        const double xn = fmin(fmin(1.0, xe + move), fmax(fmax(0.0, xe - move), S->B[e] * s));
        xnew[e] = xn;
        mx = fmax(mx, fabs(xn - xe));
        vol = fma(w[e], xn, vol);
    }
    double v[1] = {mx}, tot[1];
    if (tog::grid_reduce_last<1, true>(v, S->partials, &oc.cnt[1], tot))
        if (threadIdx.x == 0) {
            result[0] = tot[0];
            result[1] = lmid;
        }
    double v2[1] = {vol}, tot2[1];
    if (tog::grid_reduce_last<1>(v2, S->partials + 2 * kNoallocBlocks, &oc.cnt[2], tot2))
        if (threadIdx.x == 0) result[2] = tot2[0];
}

}  // namespace

extern "C" {

// Declared in include/topopt_gb300.h.
int tog_oc_update_noalloc(int64_t n, const double* x_dev, const double* dc_dev, const double* dv_dev,
                          const double* w_dev, double volfrac, double move, double* xnew_dev, double* result_dev,
                          void* stream) {
    if (n <= 0) return noalloc_fail(TOG_ERR_ARG, "tog_oc_update_noalloc: n must be > 0");
    if (n > kNoallocMaxCells)
        return noalloc_fail(TOG_ERR_ARG, "tog_oc_update_noalloc: n = " + std::to_string((long long)n) +
                                             " exceeds the static scratch capacity of " +
                                             std::to_string(kNoallocMaxCells) + " cells");
    if (!x_dev || !dc_dev || !dv_dev || !w_dev || !xnew_dev || !result_dev)
        return noalloc_fail(TOG_ERR_ARG, "tog_oc_update_noalloc: null device array");
    if (!(move > 0) || !(volfrac > 0 && volfrac <= 1))
        return noalloc_fail(TOG_ERR_ARG, "tog_oc_update_noalloc: need move > 0 and 0 < volfrac <= 1");
    NoallocScratch* S = nullptr;
    int rc = noalloc_scratch(&S);
    if (rc != TOG_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long want = (n + kNoallocThreads - 1) / kNoallocThreads;
    const int nb = (int)(want < kNoallocBlocks ? want : kNoallocBlocks);
    k_na_prep<<<nb, kNoallocThreads, 0, s>>>(x_dev, dc_dev, dv_dev, n, volfrac, move, S);
    for (int i = 0; i < kNoallocMaxSteps; ++i) k_na_step<<<nb, kNoallocThreads, 0, s>>>(x_dev, w_dev, n, S);
    k_na_final<<<nb, kNoallocThreads, 0, s>>>(x_dev, w_dev, xnew_dev, n, S, result_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(TOG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return TOG_OK;
}

}  // extern "C"
