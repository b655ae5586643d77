// Batched 2D SIMP: many independent quad4 cantilevers of uneven size advance
// one design iteration together in ONE CUDA-graph launch (tog_batch_step).
//
// Each problem keeps its own filter, FP32-IR solve (reliable updates),
// compliance and OC state; all problems' arrays are concatenated in HBM and the
// kernels walk work-item lists ((problem, tile) pairs), so one launch serves
// every problem whatever its size.  Data-dependent loops (PCG iterations, OC
// bisection) are conditional WHILE nodes of the graph whose condition the
// kernels set on the device: the host sees one graph launch per design
// iteration and reads back a few scalars.
//
// Per problem, the algorithm is the one of the single-problem path
// (tog_simp_step with TOG_FP32_IR and warm start): the references of that path
// apply (TopOpt.jl src/FEA/matrix_free_operator.jl:66-105, solvers_api.jl:177-220,
// src/Functions/compute_element_energy.jl:18-38, src/CheqFilters/density_filter.jl:
// 25-121; OC has no reference counterpart).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/topopt_gb300.h"
#include "tog_device.cuh"
#include "tog_host.h"
#include "tog_internal.h"
#include "tog_reduce.cuh"

using namespace tog;

namespace {

constexpr int kBThreads = 256;
constexpr int kNodeChunk = 1024;   // nodes per node item
constexpr int kCellChunk = 1024;   // cells per cell item
constexpr int kMvWarps = 4;        // matvec items (warps) per block
constexpr int kOcMax = 100;        // bisection step cap
constexpr int kMaxLoops = 1 << 20; // PCG loop cap of one design iteration

enum { M_PCG = 0, M_RU = 1, M_DONE = 2, M_FAIL = 3, M_INIT = 4 };

struct BProb {
    int nel[2], nn[2];
    long long noff, eoff;        // first node / cell of the problem
    int mv0, nmv;                // matvec items
    int nd0, nnd;                // node items
    int ce0, nce;                // cell items
    int s0, S;                   // filter stencil slice
    double volfrac, tol;
};

struct BState {
    PcgState pcg;                // FP32 inner PCG
    double s;                    // scale of r32 (FP64 residual norm at the last update)
    double res, best;
    int mode, stall, updates, pad;
    double comp;                 // compliance
    OcState oc;
    unsigned cnt[8];             // per-problem last-item counters
};

struct BGlobal {
    unsigned cnt[8];
    int loops, active, failed, oc_active;
};

struct Item {   // one work item
    int prob;
    int a, b;   // matvec: x tile, y chunk start; node/cell items: chunk start
};

struct BArgs {
    const BProb* P;
    BState* B;
    BGlobal* G;
    const Item* mv;
    const Item* nd;
    const Item* ce;
    int nmv, nnd, nce, nprob, LY;
    const uint8_t* fixmask;
    const double* f;
    double *u, *r64;
    float *x32, *r32, *P0, *P1, *q32, *dinv32, *e32;
    double *e64, *vars, *x, *xnew, *dc, *dv, *grad, *B_oc, *nodal, *invW;
    const int* soff;
    const double* sw;
    double* partials;           // one slot per item (x2)
    Modal<float, 2> Mf;
    Modal<double, 2> Md;
    double xmin, pen, ru_delta2, move;
    int ip, maxit;
    cudaGraphConditionalHandle h_pcg, h_oc;
};

// ---- per-problem reduction: partial per item, last item of the problem sums in order
template <int NV>
__device__ bool prob_reduce_warp(double (&v)[NV], double* partials, int item, int item0, int nitems, unsigned* counter,
                                 double (&tot)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
    unsigned last = 0;
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[(size_t)item * NV + i] = v[i];
        __threadfence();
        last = (atomicAdd(counter, 1u) == (unsigned)nitems - 1) ? 1u : 0u;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) s[i] = 0.0;
    for (int t = lane; t < nitems; t += 32)
#pragma unroll
        for (int i = 0; i < NV; ++i) s[i] += __ldcg(partials + (size_t)(item0 + t) * NV + i);
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = warp_sum(s[i]);
    if (lane == 0) *counter = 0u;
    return true;
}

template <int NV, bool MAX = false>
__device__ bool prob_reduce_block(double (&v)[NV], double* partials, int item, int item0, int nitems,
                                  unsigned* counter, double (&tot)[NV]) {
    __shared__ double sred[NV][32];
    __shared__ int amlast;
    block_reduce<NV, MAX>(v, sred);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[(size_t)item * NV + i] = v[i];
        __threadfence();
        amlast = (atomicAdd(counter, 1u) == (unsigned)nitems - 1);
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) s[i] = MAX ? -1.0e308 : 0.0;
    for (int t = threadIdx.x; t < nitems; t += blockDim.x)
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const double x = __ldcg(partials + (size_t)(item0 + t) * NV + i);
            s[i] = MAX ? fmax(s[i], x) : s[i] + x;
        }
    block_reduce<NV, MAX>(s, sred);
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = s[i];
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// the last block of the whole grid (all problems finalised); used to set graph conditions
__device__ bool grid_last(unsigned* counter) {
    __shared__ int amlast;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
        amlast = (atomicAdd(counter, 1u) == nb - 1);
    }
    __syncthreads();
    if (amlast) {
        __threadfence();
        if (threadIdx.x == 0 && threadIdx.y == 0) *counter = 0u;
    }
    return amlast;
}

__device__ __forceinline__ Dims pdims(const BProb& P) {
    Dims D;
    D.dim = 2;
    D.nel[0] = P.nel[0];
    D.nel[1] = P.nel[1];
    D.nel[2] = 1;
    D.nn[0] = P.nn[0];
    D.nn[1] = P.nn[1];
    D.nn[2] = 1;
    D.nnodes = (long long)P.nn[0] * P.nn[1];
    D.ncells = (long long)P.nel[0] * P.nel[1];
    return D;
}

// ---------------------------------------------------------------------------
// design iteration start: every problem to M_INIT, counters cleared
__global__ void bk_begin(BArgs A) {
    for (int b = threadIdx.x; b < A.nprob; b += blockDim.x) {
        A.B[b].mode = M_INIT;
        A.B[b].stall = 0;
        A.B[b].updates = 0;
        A.B[b].pcg.it = 0;
    }
    if (threadIdx.x == 0) {
        A.G->loops = 0;
        A.G->failed = 0;
    }
}

// ---- filters (per problem, node-based, as the single-problem kernels) ----
__global__ void __launch_bounds__(kBThreads) bk_filt_nodeavg(BArgs A, const double* __restrict__ xe,
                                                              double* __restrict__ nodal) {
    const Item it = A.nd[blockIdx.x];
    const BProb P = A.P[it.prob];
    const Dims D = pdims(P);
    for (int t = threadIdx.x; t < kNodeChunk; t += blockDim.x) {
        const long long n = (long long)it.a + t;
        if (n >= D.nnodes) break;
        const int ix = (int)(n % D.nn[0]), iy = (int)(n / D.nn[0]);
        double s = 0.0;
        int cnt = 0;
        for (int by = 0; by < 2; ++by)
            for (int bx = 0; bx < 2; ++bx) {
                const int cx = ix - 1 + bx, cy = iy - 1 + by;
                if (cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1]) {
                    s += xe[P.eoff + cx + (long long)D.nel[0] * cy];
                    ++cnt;
                }
            }
        nodal[P.noff + n] = cnt ? s / cnt : 0.0;
    }
}

__global__ void __launch_bounds__(kBThreads) bk_filt_nodeavgT(BArgs A, const double* __restrict__ nodal,
                                                               double* __restrict__ out) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    const Dims D = pdims(P);
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= D.ncells) break;
        const int ex = (int)(e % D.nel[0]), ey = (int)(e / D.nel[0]);
        double s = 0.0;
        for (int j = 0; j < 4; ++j) {
            const int ix = ex + (j & 1), iy = ey + (j >> 1);
            s += nodal[P.noff + ix + (long long)D.nn[0] * iy] / valence<2>(ix, iy, 0, D);
        }
        out[P.eoff + e] = s;
    }
}

__global__ void __launch_bounds__(kBThreads) bk_filt_invW(BArgs A) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    const Dims D = pdims(P);
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= D.ncells) break;
        const int ex = (int)(e % D.nel[0]), ey = (int)(e / D.nel[0]);
        double W = 0.0;
        for (int s = P.s0; s < P.s0 + P.S; ++s) {
            const int ix = ex + A.soff[3 * s], iy = ey + A.soff[3 * s + 1];
            if (ix >= 0 && ix < D.nn[0] && iy >= 0 && iy < D.nn[1]) W += A.sw[s] * valence<2>(ix, iy, 0, D);
        }
        A.invW[P.eoff + e] = W > 0.0 ? 1.0 / W : 0.0;
    }
}

__global__ void __launch_bounds__(kBThreads) bk_filt_cone(BArgs A, const double* __restrict__ nodal,
                                                           const double* __restrict__ xin, double* __restrict__ ye) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    const Dims D = pdims(P);
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= D.ncells) break;
        const int ex = (int)(e % D.nel[0]), ey = (int)(e / D.nel[0]);
        double s_ = 0.0;
        for (int s = P.s0; s < P.s0 + P.S; ++s) {
            const int ix = ex + A.soff[3 * s], iy = ey + A.soff[3 * s + 1];
            if (ix >= 0 && ix < D.nn[0] && iy >= 0 && iy < D.nn[1])
                s_ += A.sw[s] * valence<2>(ix, iy, 0, D) * nodal[P.noff + ix + (long long)D.nn[0] * iy];
        }
        const double iw = A.invW[P.eoff + e];
        ye[P.eoff + e] = iw > 0.0 ? s_ * iw : xin[P.eoff + e];
    }
}

__global__ void __launch_bounds__(kBThreads) bk_filt_coneT(BArgs A, const double* __restrict__ de,
                                                            double* __restrict__ nodal) {
    const Item it = A.nd[blockIdx.x];
    const BProb P = A.P[it.prob];
    const Dims D = pdims(P);
    for (int t = threadIdx.x; t < kNodeChunk; t += blockDim.x) {
        const long long n = (long long)it.a + t;
        if (n >= D.nnodes) break;
        const int ix = (int)(n % D.nn[0]), iy = (int)(n / D.nn[0]);
        double s_ = 0.0;
        for (int s = P.s0; s < P.s0 + P.S; ++s) {
            const int ex = ix - A.soff[3 * s], ey = iy - A.soff[3 * s + 1];
            if (ex >= 0 && ex < D.nel[0] && ey >= 0 && ey < D.nel[1]) {
                const long long e = P.eoff + ex + (long long)D.nel[0] * ey;
                s_ += A.sw[s] * A.invW[e] * de[e];
            }
        }
        nodal[P.noff + n] = s_ * valence<2>(ix, iy, 0, D);
    }
}

// ---- densities -> element scales, Jacobi diagonal ----
__global__ void __launch_bounds__(kBThreads) bk_escale(BArgs A) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    const long long nc = (long long)P.nel[0] * P.nel[1];
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= nc) break;
        const double v = fma(ipow(A.vars[P.eoff + e], A.pen, A.ip), 1.0 - A.xmin, A.xmin);
        A.e64[P.eoff + e] = v;
        A.e32[P.eoff + e] = (float)v;
    }
}

__global__ void __launch_bounds__(kBThreads) bk_nodesum(BArgs A) {
    const Item it = A.nd[blockIdx.x];
    const BProb P = A.P[it.prob];
    const Dims D = pdims(P);
    for (int t = threadIdx.x; t < kNodeChunk; t += blockDim.x) {
        const long long n = (long long)it.a + t;
        if (n >= D.nnodes) break;
        const int ix = (int)(n % D.nn[0]), iy = (int)(n / D.nn[0]);
        double s = 0.0;
        for (int by = 0; by < 2; ++by)
            for (int bx = 0; bx < 2; ++bx) {
                const int cx = ix - 1 + bx, cy = iy - 1 + by;
                if (cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1]) s += A.e64[P.eoff + cx + (long long)D.nel[0] * cy];
            }
        A.dinv32[P.noff + n] = s > 0.0 ? (float)(1.0 / s) : 0.f;
    }
}

// ---------------------------------------------------------------------------
// matrix-free operator over matvec items: one warp = 32 element columns (31
// owned node columns) of one problem, marching LY element rows in y.
//   MV_PCG (FP32): p = D^-1 r + beta p_old, q = K p, p.q -> alpha  (mode M_PCG)
//   MV_RESID (FP64): r64 = f - K (u + s x32), ||r64||^2 -> decision (modes M_INIT / M_RU)
template <typename T, int MODE>
__global__ void __launch_bounds__(32 * kMvWarps) bk_matvec(BArgs A) {
    const int lane = threadIdx.x & 31;
    const int item = blockIdx.x * kMvWarps + (threadIdx.x >> 5);
    if (item >= A.nmv) return;
    const Item it = A.mv[item];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    const int mode = S.mode;
    if (MODE == MV_PCG && mode != M_PCG) return;
    if (MODE == MV_RESID && mode != M_INIT && mode != M_RU) return;
    const int nelx = P.nel[0], nely = P.nel[1], nnx = P.nn[0], nny = P.nn[1];
    const int ex = 31 * it.a - 1 + lane;
    const int ky0 = it.b;
    const bool own_x = lane >= 1 && ex < nnx;
    T beta = T(0);
    const float* pold = nullptr;
    float* pnew = nullptr;
    double sc = 0.0;
    if (MODE == MV_PCG) {
        const int itn = S.pcg.it;
        pnew = (itn & 1) ? A.P1 : A.P0;
        pold = (itn & 1) ? A.P0 : A.P1;
        beta = (T)S.pcg.beta;
    } else {
        sc = (mode == M_RU) ? S.s : 0.0;
    }
    const Modal<T, 2>& M = *reinterpret_cast<const Modal<T, 2>*>(sizeof(T) == 4 ? (const void*)&A.Mf : (const void*)&A.Md);
    auto load_row = [&](int kk, T (&v)[2][2]) {
#pragma unroll
        for (int bx = 0; bx < 2; ++bx) {
            const int ix = ex + bx;
            v[0][bx] = v[1][bx] = T(0);
            if (ix >= 0 && ix < nnx && kk >= 0 && kk < nny) {
                const long long n = P.noff + ix + (long long)nnx * kk;
                if (MODE == MV_PCG) {
                    const float d = A.dinv32[n];
#pragma unroll
                    for (int c = 0; c < 2; ++c)
                        v[c][bx] = (T)fmaf((float)beta, pold[2 * n + c], d * A.Mf.kdinv[c] * A.r32[2 * n + c]);
                } else {
                    const unsigned m = A.fixmask[n];
#pragma unroll
                    for (int c = 0; c < 2; ++c)
                        v[c][bx] = ((m >> c) & 1u) ? T(0) : (T)(A.u[2 * n + c] + sc * (double)A.x32[2 * n + c]);
                }
            }
        }
    };
    T lo[2][2], up[2][2];
    load_row(ky0 - 1, lo);
    T carry[2] = {T(0), T(0)};
    double acc = 0.0;
    const int kend = min(ky0 + A.LY - 1, nely);
    for (int k = ky0 - 1; k <= kend; ++k) {
        load_row(k + 1, up);
        T y[2][4];
        const bool inel = ex >= 0 && ex < nelx && k >= 0 && k < nely;
        if (inel) {
            const T rho = (T)(sizeof(T) == 4 ? (double)A.e32[P.eoff + ex + (long long)nelx * k]
                                             : A.e64[P.eoff + ex + (long long)nelx * k]);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                y[c][0] = lo[c][0];
                y[c][1] = lo[c][1];
                y[c][2] = up[c][0];
                y[c][3] = up[c][1];
            }
            element_apply<T, 2>(M, rho, y);
        } else {
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int j = 0; j < 4; ++j) y[c][j] = T(0);
        }
        T col[2][2];
#pragma unroll
        for (int by = 0; by < 2; ++by)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const T t = __shfl_up_sync(0xffffffffu, y[c][1 + 2 * by], 1);
                col[c][by] = y[c][2 * by] + (lane > 0 ? t : T(0));
            }
        if (k >= ky0 && own_x && k < nny) {
            const long long n = P.noff + ex + (long long)nnx * k;
            const unsigned m = A.fixmask[n];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const T tot = carry[c] + col[c][0];
                if (MODE == MV_PCG) {
                    const T pv = lo[c][0];
                    const T qv = ((m >> c) & 1u) ? T(0) : tot;
                    pnew[2 * n + c] = (float)pv;
                    A.q32[2 * n + c] = (float)qv;
                    acc += (double)pv * (double)qv;
                } else {
                    const double rv = ((m >> c) & 1u) ? 0.0 : A.f[2 * n + c] - (double)tot;
                    A.r64[2 * n + c] = rv;
                    acc += rv * rv;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            carry[c] = col[c][1];
            lo[c][0] = up[c][0];
            lo[c][1] = up[c][1];
        }
    }
    double v[1] = {acc}, tot[1];
    if (prob_reduce_warp<1>(v, A.partials, item, P.mv0, P.nmv, &S.cnt[MODE == MV_PCG ? 0 : 1], tot)) {
        if (lane == 0) {
            if (MODE == MV_PCG) {
                S.pcg.pq = tot[0];
                if (!(tot[0] > 0.0) || !isfinite(tot[0]))
                    S.mode = M_RU;   // breakdown: refresh from the true residual
                else
                    S.pcg.alpha = S.pcg.rz / tot[0];
            } else {
                const double res = sqrt(tot[0]);
                S.res = res;
                if (!isfinite(res)) {
                    S.mode = M_FAIL;
                } else if (res <= P.tol) {
                    S.mode = (mode == M_RU) ? M_RU : M_DONE;   // M_RU: the rescale pass applies the last correction
                    S.stall = -1;                                // converged marker for the rescale pass
                } else if (mode == M_RU) {
                    if (res < 0.5 * S.best) {
                        S.best = res;
                        S.stall = 0;
                    } else if (++S.stall >= 8) {
                        S.mode = M_FAIL;
                    }
                } else {
                    S.best = res;
                }
            }
        }
    }
}

// Reliable update / initialisation over node items (problems in M_INIT or M_RU):
// u += s x32; then, unless converged, r32 = r64 / res, x32 = 0, the last
// direction rescaled (M_RU) or cleared (M_INIT), and the PCG scalars rebuilt.
// The last block of the grid sets the PCG-loop condition.
__global__ void __launch_bounds__(kBThreads) bk_rescale(BArgs A) {
    const Item it = A.nd[blockIdx.x];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    const int mode = S.mode;
    const bool act = (mode == M_INIT || mode == M_RU);
    const bool conv = act && S.stall == -1;
    double v[2] = {0.0, 0.0};
    if (act) {
        const long long nnodes = (long long)P.nn[0] * P.nn[1];
        const double s_old = (mode == M_RU) ? S.s : 0.0;
        const double res = S.res;
        const double inv = res > 0.0 ? 1.0 / res : 0.0;
        const int itn = S.pcg.it;
        float* plast = ((itn - 1) & 1) ? A.P1 : A.P0;
        const float ratio = (float)(res > 0.0 ? s_old / res : 0.0);
        float arz = 0.f, arr = 0.f;
        for (int t = threadIdx.x; t < kNodeChunk; t += blockDim.x) {
            const long long nl = (long long)it.a + t;
            if (nl >= nnodes) break;
            const long long n = P.noff + nl;
            const float d = A.dinv32[n];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const long long i = 2 * n + c;
                if (mode == M_RU) A.u[i] = fma(s_old, (double)A.x32[i], A.u[i]);
                if (!conv) {
                    const float rn = (float)(A.r64[i] * inv);
                    A.r32[i] = rn;
                    A.x32[i] = 0.f;
                    if (mode == M_RU) {
                        plast[i] *= ratio;
                    } else {
                        A.P0[i] = 0.f;
                        A.P1[i] = 0.f;
                    }
                    arz = fmaf(rn, d * A.Mf.kdinv[c] * rn, arz);
                    arr = fmaf(rn, rn, arr);
                }
            }
        }
        v[0] = arz;
        v[1] = arr;
        double tot[2];
        if (prob_reduce_block<2>(v, A.partials, blockIdx.x, P.nd0, P.nnd, &S.cnt[2], tot)) {
            if (threadIdx.x == 0) {
                if (conv) {
                    S.mode = M_DONE;
                } else {
                    if (mode == M_RU) {
                        const double q = s_old / res;
                        const double rz_prev = S.pcg.rz_old * q * q;
                        S.pcg.beta = rz_prev > 0.0 ? tot[0] / rz_prev : 0.0;
                        S.updates += 1;
                    } else {
                        S.pcg.beta = 0.0;
                        S.pcg.it = 0;
                    }
                    S.pcg.rz = tot[0];
                    S.pcg.rr = tot[1];
                    S.pcg.rr_max = tot[1];
                    S.pcg.tol2 = (P.tol / res) * (P.tol / res);
                    S.pcg.ru_delta2 = A.ru_delta2;
                    S.pcg.maxit = A.maxit;
                    S.s = res;
                    S.stall = (mode == M_RU) ? S.stall : 0;
                    S.mode = (S.pcg.it >= A.maxit) ? M_FAIL : M_PCG;
                }
            }
        }
    }
    if (grid_last(&A.G->cnt[0])) {
        if (threadIdx.x == 0) {
            int active = 0, failed = 0;
            for (int b = 0; b < A.nprob; ++b) {
                const int m = A.B[b].mode;
                active += (m == M_PCG || m == M_RU);
                failed += (m == M_FAIL);
            }
            A.G->loops += 1;
            A.G->active = active;
            A.G->failed = failed;
            cudaGraphSetConditional(A.h_pcg, (active > 0 && A.G->loops < kMaxLoops) ? 1u : 0u);
        }
    }
}

// PCG update over node items (M_PCG problems): x += alpha p, r -= alpha q, r.z, r.r
__global__ void __launch_bounds__(kBThreads) bk_update(BArgs A) {
    const Item it = A.nd[blockIdx.x];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    if (S.mode != M_PCG) return;
    const int itn = S.pcg.it;
    const float* __restrict__ p = (itn & 1) ? A.P1 : A.P0;
    const float alpha = (float)S.pcg.alpha;
    const long long nnodes = (long long)P.nn[0] * P.nn[1];
    float arz = 0.f, arr = 0.f;
    for (int t = threadIdx.x; t < kNodeChunk; t += blockDim.x) {
        const long long nl = (long long)it.a + t;
        if (nl >= nnodes) break;
        const long long n = P.noff + nl;
        const float d = A.dinv32[n];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const long long i = 2 * n + c;
            A.x32[i] = fmaf(alpha, p[i], A.x32[i]);
            const float rn = fmaf(-alpha, A.q32[i], A.r32[i]);
            A.r32[i] = rn;
            arz = fmaf(rn, d * A.Mf.kdinv[c] * rn, arz);
            arr = fmaf(rn, rn, arr);
        }
    }
    double v[2] = {arz, arr}, tot[2];
    if (prob_reduce_block<2>(v, A.partials, blockIdx.x, P.nd0, P.nnd, &S.cnt[3], tot)) {
        if (threadIdx.x == 0) {
            PcgState& st = S.pcg;
            const double rzo = st.rz;
            st.rz_old = rzo;
            st.rz = tot[0];
            st.beta = rzo != 0.0 ? tot[0] / rzo : 0.0;
            st.rr = tot[1];
            st.it = itn + 1;
            if (!isfinite(tot[1]) || tot[1] <= st.tol2 || tot[1] < st.ru_delta2 * st.rr_max)
                S.mode = M_RU;
            else if (itn + 1 >= st.maxit)
                S.mode = M_RU;   // the update pass decides (fails when maxit is spent)
            st.rr_max = fmax(st.rr_max, tot[1]);
        }
    }
}

// ---- compliance + sensitivities (FP64, cell items) ----
__global__ void __launch_bounds__(kBThreads) bk_compliance(BArgs A) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    const Dims D = pdims(P);
    double acc = 0.0;
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= D.ncells) break;
        const int ex = (int)(e % D.nel[0]), ey = (int)(e / D.nel[0]);
        double uc[2][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long n = P.noff + (ex + (j & 1)) + (long long)D.nn[0] * (ey + (j >> 1));
            uc[0][j] = A.u[2 * n];
            uc[1][j] = A.u[2 * n + 1];
        }
        const double ce = element_energy<2>(A.Md, uc);
        const double x = A.vars[P.eoff + e];
        const double rho = fma(ipow(x, A.pen, A.ip), 1.0 - A.xmin, A.xmin);
        const double drho = (1.0 - A.xmin) * A.pen * (A.pen == 0.0 ? 0.0 : ipow(x, A.pen - 1.0, A.ip > 0 ? A.ip - 1 : -1));
        A.grad[P.eoff + e] = -drho * ce;
        acc = fma(rho, ce, acc);
    }
    double v[1] = {acc}, tot[1];
    if (prob_reduce_block<1>(v, A.partials, blockIdx.x, P.ce0, P.nce, &S.cnt[4], tot))
        if (threadIdx.x == 0) S.comp = tot[0];
}

// ---- OC (cell items) ----
__global__ void __launch_bounds__(kBThreads) bk_oc_prep(BArgs A) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    const long long nc = (long long)P.nel[0] * P.nel[1];
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= nc) break;
        const long long g = P.eoff + e;
        A.B_oc[g] = A.x[g] * sqrt(fmax(0.0, -A.dc[g]) / A.dv[g]);
    }
    if (it.a == 0 && threadIdx.x == 0) {
        S.oc.l1 = 0.0;
        S.oc.l2 = 1e9;
        S.oc.tol = 1e-3;
        S.oc.target = P.volfrac;
        S.oc.move = A.move;
        S.oc.steps = 0;
        S.oc.done = 0;
        S.oc.maxsteps = kOcMax;
    }
}

__global__ void __launch_bounds__(kBThreads) bk_oc_step(BArgs A) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    if (!S.oc.done) {
        const double lmid = 0.5 * (S.oc.l2 + S.oc.l1), s = 1.0 / sqrt(lmid), move = S.oc.move;
        const long long nc = (long long)P.nel[0] * P.nel[1];
        double acc = 0.0;
        for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
            const long long e = (long long)it.a + t;
            if (e >= nc) break;
            const long long g = P.eoff + e;
            const double xe = A.x[g];
            const double xn = fmin(fmin(1.0, xe + move), fmax(fmax(0.0, xe - move), A.B_oc[g] * s));
            acc = fma(A.dv[g], xn, acc);
        }
        double v[1] = {acc}, tot[1];
        if (prob_reduce_block<1>(v, A.partials, blockIdx.x, P.ce0, P.nce, &S.cnt[5], tot)) {
            if (threadIdx.x == 0) {
                S.oc.vol = tot[0];
                if (tot[0] > S.oc.target)
                    S.oc.l1 = lmid;
                else
                    S.oc.l2 = lmid;
                S.oc.steps += 1;
                if ((S.oc.l2 - S.oc.l1) / (S.oc.l1 + S.oc.l2) <= S.oc.tol || S.oc.steps >= S.oc.maxsteps) S.oc.done = 1;
            }
        }
    }
    if (grid_last(&A.G->cnt[1])) {
        if (threadIdx.x == 0) {
            int act = 0;
            for (int b = 0; b < A.nprob; ++b) act += !A.B[b].oc.done;
            A.G->oc_active = act;
            cudaGraphSetConditional(A.h_oc, act > 0 ? 1u : 0u);
        }
    }
}

__global__ void __launch_bounds__(kBThreads) bk_oc_final(BArgs A) {
    const Item it = A.ce[blockIdx.x];
    const BProb P = A.P[it.prob];
    BState& S = A.B[it.prob];
    const double lmid = 0.5 * (S.oc.l2 + S.oc.l1), s = 1.0 / sqrt(lmid), move = S.oc.move;
    const long long nc = (long long)P.nel[0] * P.nel[1];
    double mx = 0.0;
    for (int t = threadIdx.x; t < kCellChunk; t += blockDim.x) {
        const long long e = (long long)it.a + t;
        if (e >= nc) break;
        const long long g = P.eoff + e;
        const double xe = A.x[g];
        const double xn = fmin(fmin(1.0, xe + move), fmax(fmax(0.0, xe - move), A.B_oc[g] * s));
        A.xnew[g] = xn;
        mx = fmax(mx, fabs(xn - xe));
    }
    double v[1] = {mx}, tot[1];
    if (prob_reduce_block<1, true>(v, A.partials, blockIdx.x, P.ce0, P.nce, &S.cnt[6], tot)) {
        if (threadIdx.x == 0) {
            S.oc.change = tot[0];
            S.oc.lmid = lmid;
        }
    }
}

__global__ void __launch_bounds__(kBThreads) bk_copy(double* __restrict__ dst, const double* __restrict__ src,
                                                     long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

}  // namespace

struct tog_batch {
    int nprob = 0;
    std::vector<BProb> probs;
    std::vector<Item> mv, nd, ce;
    long long nnodes = 0, ncells = 0;
    int LY = 32;
    double xmin = 1e-9, pen = 3.0, rtol = 1e-8, move = 0.2;
    int maxit = 1 << 20;
    cudaStream_t own = nullptr, stream = nullptr;
    int nsm = 152;
    // device
    BProb* d_P = nullptr;
    BState* d_B = nullptr;
    BGlobal* d_G = nullptr;
    Item *d_mv = nullptr, *d_nd = nullptr, *d_ce = nullptr;
    std::vector<void*> allocs;
    BArgs A{};
    std::vector<BState> h_B;
    BGlobal* h_G = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle h_pcg{}, h_oc{};
    int steps = 0;
};

namespace {

int bfail(int code, const std::string& m) { return tog::set_error(code, m.c_str()); }

#define TB_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return bfail(e_ == cudaErrorMemoryAllocation ? TOG_ERR_OOM : TOG_ERR_CUDA,                 \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

template <typename T>
int balloc(tog_batch* b, T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T) + 16);
    if (e != cudaSuccess) return bfail(TOG_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b->allocs.push_back(*p);
    return TOG_OK;
}

void build_mv_items(tog_batch* b, int LY) {
    b->mv.clear();
    for (int p = 0; p < b->nprob; ++p) {
        BProb& P = b->probs[p];
        P.mv0 = (int)b->mv.size();
        const int tx = (P.nn[0] + 30) / 31;
        const int ty = (P.nn[1] + LY - 1) / LY;
        for (int y = 0; y < ty; ++y)
            for (int x = 0; x < tx; ++x) b->mv.push_back(Item{p, x, y * LY});
        P.nmv = (int)b->mv.size() - P.mv0;
    }
}

// record the whole design iteration into b->graph (kernels + two conditional WHILE nodes)
int build_graph(tog_batch* b) {
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    TB_CUDA(cudaGraphCreate(&b->graph, 0));
    TB_CUDA(cudaGraphConditionalHandleCreate(&b->h_pcg, b->graph, 0, cudaGraphCondAssignDefault));
    TB_CUDA(cudaGraphConditionalHandleCreate(&b->h_oc, b->graph, 1, cudaGraphCondAssignDefault));
    b->A.h_pcg = b->h_pcg;
    b->A.h_oc = b->h_oc;
    const BArgs A = b->A;
    cudaStream_t s = b->own;
    const int nmvb = (b->A.nmv + kMvWarps - 1) / kMvWarps;
    const int nce = b->A.nce, nnd = b->A.nnd;
    auto tail = [&](std::vector<cudaGraphNode_t>& deps) -> int {
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        TB_CUDA(cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &d, nullptr, &nd));
        deps.assign(d, d + nd);
        return TOG_OK;
    };
    std::vector<cudaGraphNode_t> deps;
    // segment 1: filter, scales, initial FP64 residual and PCG set-up
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, b->graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    bk_begin<<<1, 256, 0, s>>>(A);
    bk_filt_nodeavg<<<nnd, kBThreads, 0, s>>>(A, A.x, A.nodal);
    bk_filt_cone<<<nce, kBThreads, 0, s>>>(A, A.nodal, A.x, A.vars);
    bk_escale<<<nce, kBThreads, 0, s>>>(A);
    bk_nodesum<<<nnd, kBThreads, 0, s>>>(A);
    bk_matvec<double, MV_RESID><<<nmvb, 32 * kMvWarps, 0, s>>>(A);
    bk_rescale<<<nnd, kBThreads, 0, s>>>(A);
    {
        int rc = tail(deps);
        if (rc != TOG_OK) return rc;
    }
    cudaGraph_t g1;
    TB_CUDA(cudaStreamEndCapture(s, &g1));
    // PCG WHILE loop
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = b->h_pcg;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wpcg;
    TB_CUDA(cudaGraphAddNode(&wpcg, b->graph, deps.data(), nullptr, deps.size(), &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    bk_matvec<float, MV_PCG><<<nmvb, 32 * kMvWarps, 0, s>>>(A);
    bk_update<<<nnd, kBThreads, 0, s>>>(A);
    bk_matvec<double, MV_RESID><<<nmvb, 32 * kMvWarps, 0, s>>>(A);
    bk_rescale<<<nnd, kBThreads, 0, s>>>(A);
    cudaGraph_t gb;
    TB_CUDA(cudaStreamEndCapture(s, &gb));
    // segment 2: compliance, filter pullback, OC prep
    cudaGraphNode_t d1[1] = {wpcg};
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, b->graph, d1, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    bk_compliance<<<nce, kBThreads, 0, s>>>(A);
    bk_filt_coneT<<<nnd, kBThreads, 0, s>>>(A, A.grad, A.nodal);
    bk_filt_nodeavgT<<<nce, kBThreads, 0, s>>>(A, A.nodal, A.dc);
    bk_oc_prep<<<nce, kBThreads, 0, s>>>(A);
    {
        int rc = tail(deps);
        if (rc != TOG_OK) return rc;
    }
    cudaGraph_t g2;
    TB_CUDA(cudaStreamEndCapture(s, &g2));
    cudaGraphNodeParams co{};
    co.type = cudaGraphNodeTypeConditional;
    co.conditional.handle = b->h_oc;
    co.conditional.type = cudaGraphCondTypeWhile;
    co.conditional.size = 1;
    cudaGraphNode_t woc;
    TB_CUDA(cudaGraphAddNode(&woc, b->graph, deps.data(), nullptr, deps.size(), &co));
    cudaGraph_t obody = co.conditional.phGraph_out[0];
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, obody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    bk_oc_step<<<nce, kBThreads, 0, s>>>(A);
    cudaGraph_t gob;
    TB_CUDA(cudaStreamEndCapture(s, &gob));
    cudaGraphNode_t d2[1] = {woc};
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, b->graph, d2, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    bk_oc_final<<<nce, kBThreads, 0, s>>>(A);
    bk_copy<<<b->nsm * 4, kBThreads, 0, s>>>(A.x, A.xnew, b->ncells);
    cudaGraph_t g3;
    TB_CUDA(cudaStreamEndCapture(s, &g3));
    TB_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return TOG_OK;
}

}  // namespace

extern "C" {

int tog_batch_create(int32_t nprob, const int32_t* nelx, const int32_t* nely, const int32_t* load_j,
                     const double* volfrac, const double* rmin, const tog_problem_desc* material, double rtol,
                     int32_t maxiter, tog_batch** out) {
    if (!out || nprob <= 0 || !nelx || !nely || !load_j || !volfrac || !rmin || !material)
        return bfail(TOG_ERR_ARG, "tog_batch_create: bad arguments");
    *out = nullptr;
    if (material->dim != 2) return bfail(TOG_ERR_ARG, "tog_batch_create: batches are 2D (quad4)");
    tog_batch* b = new tog_batch();
    b->nprob = nprob;
    b->xmin = material->xmin;
    b->pen = material->penalty;
    b->rtol = rtol;
    b->maxit = maxiter > 0 ? maxiter : (1 << 20);
    // element operator (identical for every problem: same element size and material)
    double Ke[64], kd[2];
    element_stiffness(2, material->size, material->E, material->nu, material->plane_stress, Ke);
    Modal<double, 2> Md{};
    Modal<float, 2> Mf{};
    try {
        modal_operator(2, Ke, &Md.D[0][0], &Md.O[0][0][0], kd);
    } catch (const std::exception& ex) {
        delete b;
        return bfail(TOG_ERR_ARG, ex.what());
    }
    for (int m = 0; m < 4; ++m)
        for (int c = 0; c < 2; ++c) {
            Mf.D[m][c] = (float)Md.D[m][c];
            for (int d = 0; d < 2; ++d) Mf.O[m][c][d] = (float)Md.O[m][c][d];
        }
    for (int c = 0; c < 2; ++c) {
        Md.kdinv[c] = 1.0 / kd[c];
        Mf.kdinv[c] = (float)(1.0 / kd[c]);
    }
    // problems, items, stencils, boundary conditions and loads
    std::vector<int> soff;
    std::vector<double> sw;
    b->probs.resize(nprob);
    long long noff = 0, eoff = 0;
    for (int p = 0; p < nprob; ++p) {
        if (nelx[p] < 1 || nely[p] < 1 || load_j[p] < 0 || load_j[p] > nely[p] || !(volfrac[p] > 0 && volfrac[p] <= 1) ||
            !(rmin[p] > 0)) {
            delete b;
            return bfail(TOG_ERR_ARG, "tog_batch_create: bad problem " + std::to_string(p));
        }
        BProb& P = b->probs[p];
        P.nel[0] = nelx[p];
        P.nel[1] = nely[p];
        P.nn[0] = nelx[p] + 1;
        P.nn[1] = nely[p] + 1;
        P.noff = noff;
        P.eoff = eoff;
        P.volfrac = volfrac[p];
        noff += (long long)P.nn[0] * P.nn[1];
        eoff += (long long)P.nel[0] * P.nel[1];
        std::vector<int> o;
        std::vector<double> w;
        const int S = filter_stencil(2, material->size, rmin[p], o, w);
        if (S == 0) {
            delete b;
            return bfail(TOG_ERR_ARG, "tog_batch_create: rmin of problem " + std::to_string(p) + " below the element size");
        }
        P.s0 = (int)sw.size();
        P.S = S;
        soff.insert(soff.end(), o.begin(), o.end());
        sw.insert(sw.end(), w.begin(), w.end());
        P.nd0 = (int)b->nd.size();
        for (long long n = 0; n < (long long)P.nn[0] * P.nn[1]; n += kNodeChunk) b->nd.push_back(Item{p, (int)n, 0});
        P.nnd = (int)b->nd.size() - P.nd0;
        P.ce0 = (int)b->ce.size();
        for (long long e = 0; e < (long long)P.nel[0] * P.nel[1]; e += kCellChunk) b->ce.push_back(Item{p, (int)e, 0});
        P.nce = (int)b->ce.size() - P.ce0;
        P.tol = rtol * 1.0;   // |f| = 1 (unit load)
    }
    b->nnodes = noff;
    b->ncells = eoff;
    build_mv_items(b, b->LY);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return bfail(TOG_ERR_CUDA, "stream creation failed");
    }
    b->stream = b->own;
    BArgs& A = b->A;
    const long long NN = b->nnodes, NC = b->ncells;
    int rc = TOG_OK;
    auto R = [&](int r) {
        if (rc == TOG_OK) rc = r;
    };
    uint8_t* fixmask = nullptr;
    double* f = nullptr;
    int* d_soff = nullptr;
    double* d_sw = nullptr;
    R(balloc(b, &b->d_P, nprob));
    R(balloc(b, &b->d_B, nprob));
    R(balloc(b, &b->d_G, 1));
    R(balloc(b, &b->d_mv, b->mv.size() + 4 * 64));
    R(balloc(b, &b->d_nd, b->nd.size()));
    R(balloc(b, &b->d_ce, b->ce.size()));
    R(balloc(b, &fixmask, NN));
    R(balloc(b, &f, 2 * NN));
    R(balloc(b, &A.u, 2 * NN));
    R(balloc(b, &A.r64, 2 * NN));
    R(balloc(b, &A.x32, 2 * NN));
    R(balloc(b, &A.r32, 2 * NN));
    R(balloc(b, &A.P0, 2 * NN));
    R(balloc(b, &A.P1, 2 * NN));
    R(balloc(b, &A.q32, 2 * NN));
    R(balloc(b, &A.dinv32, NN));
    R(balloc(b, &A.nodal, NN));
    R(balloc(b, &A.e32, NC));
    R(balloc(b, &A.e64, NC));
    R(balloc(b, &A.vars, NC));
    R(balloc(b, &A.x, NC));
    R(balloc(b, &A.xnew, NC));
    R(balloc(b, &A.dc, NC));
    R(balloc(b, &A.dv, NC));
    R(balloc(b, &A.grad, NC));
    R(balloc(b, &A.B_oc, NC));
    R(balloc(b, &A.invW, NC));
    R(balloc(b, &d_soff, soff.size()));
    R(balloc(b, &d_sw, sw.size()));
    const size_t nitems = std::max(b->mv.size() + 4 * 64, std::max(b->nd.size(), b->ce.size()));
    R(balloc(b, &A.partials, 2 * nitems + 64));
    if (rc != TOG_OK) {
        std::string m = tog_last_error();
        tog_batch_destroy(b);
        bfail(rc, m);
        return rc;
    }
    // host-side masks and loads: left edge clamped, unit load [0, -1] at (nelx, load_j)
    std::vector<uint8_t> hm(NN, 0);
    std::vector<double> hf(2 * NN, 0.0);
    for (int p = 0; p < nprob; ++p) {
        const BProb& P = b->probs[p];
        for (int j = 0; j < P.nn[1]; ++j) hm[P.noff + (long long)P.nn[0] * j] = 3;
        hf[2 * (P.noff + P.nel[0] + (long long)P.nn[0] * load_j[p]) + 1] = -1.0;
    }
    A.P = b->d_P;
    A.B = b->d_B;
    A.G = b->d_G;
    A.mv = b->d_mv;
    A.nd = b->d_nd;
    A.ce = b->d_ce;
    A.nmv = (int)b->mv.size();
    A.nnd = (int)b->nd.size();
    A.nce = (int)b->ce.size();
    A.nprob = nprob;
    A.LY = b->LY;
    A.fixmask = fixmask;
    A.f = f;
    A.soff = d_soff;
    A.sw = d_sw;
    A.Mf = Mf;
    A.Md = Md;
    A.xmin = b->xmin;
    A.pen = b->pen;
    const double ipf = std::floor(b->pen);
    A.ip = (b->pen == ipf && b->pen >= 0 && b->pen <= 8) ? (int)ipf : -1;
    A.ru_delta2 = 0.01;
    A.move = b->move;
    A.maxit = b->maxit;
    cudaError_t e = cudaSuccess;
    auto C = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    C(cudaMemcpyAsync(b->d_P, b->probs.data(), nprob * sizeof(BProb), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(b->d_mv, b->mv.data(), b->mv.size() * sizeof(Item), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(b->d_nd, b->nd.data(), b->nd.size() * sizeof(Item), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(b->d_ce, b->ce.data(), b->ce.size() * sizeof(Item), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(fixmask, hm.data(), NN, cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(f, hf.data(), 2 * NN * sizeof(double), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(d_soff, soff.data(), soff.size() * sizeof(int), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(d_sw, sw.data(), sw.size() * sizeof(double), cudaMemcpyHostToDevice, b->own));
    C(cudaMemsetAsync(b->d_B, 0, nprob * sizeof(BState), b->own));
    C(cudaMemsetAsync(b->d_G, 0, sizeof(BGlobal), b->own));
    C(cudaMemsetAsync(A.u, 0, 2 * NN * sizeof(double), b->own));
    C(cudaMemsetAsync(A.x32, 0, 2 * NN * sizeof(float), b->own));
    C(cudaMemsetAsync(A.P0, 0, 2 * NN * sizeof(float), b->own));
    C(cudaMemsetAsync(A.P1, 0, 2 * NN * sizeof(float), b->own));
    C(cudaMemsetAsync(A.r32, 0, 2 * NN * sizeof(float), b->own));
    C(cudaMemsetAsync(A.q32, 0, 2 * NN * sizeof(float), b->own));
    C(cudaMemsetAsync(A.dinv32, 0, NN * sizeof(float), b->own));
    C(cudaMemsetAsync(A.e32, 0, NC * sizeof(float), b->own));
    // initial design: uniform volume fraction per problem; dv = J' (1/n) per problem
    std::vector<double> hx(NC), hinv(NC);
    for (int p = 0; p < nprob; ++p) {
        const BProb& P = b->probs[p];
        const long long nc = (long long)P.nel[0] * P.nel[1];
        for (long long i = 0; i < nc; ++i) {
            hx[P.eoff + i] = P.volfrac;
            hinv[P.eoff + i] = 1.0 / (double)nc;
        }
    }
    C(cudaMemcpyAsync(A.x, hx.data(), NC * sizeof(double), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(A.grad, hinv.data(), NC * sizeof(double), cudaMemcpyHostToDevice, b->own));
    if (e == cudaSuccess) {
        bk_filt_invW<<<A.nce, kBThreads, 0, b->own>>>(A);
        bk_filt_coneT<<<A.nnd, kBThreads, 0, b->own>>>(A, A.grad, A.nodal);
        bk_filt_nodeavgT<<<A.nce, kBThreads, 0, b->own>>>(A, A.nodal, A.dv);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->own);
    if (e == cudaSuccess && cudaHostAlloc((void**)&b->h_G, sizeof(BGlobal), cudaHostAllocDefault) != cudaSuccess)
        e = cudaErrorMemoryAllocation;
    if (e != cudaSuccess) {
        tog_batch_destroy(b);
        return bfail(TOG_ERR_CUDA, std::string("batch init: ") + cudaGetErrorString(e));
    }
    b->h_B.resize(nprob);
    rc = build_graph(b);
    if (rc != TOG_OK) {
        std::string m = tog_last_error();
        tog_batch_destroy(b);
        bfail(rc, m);
        return rc;
    }
    *out = b;
    return TOG_OK;
}

int tog_batch_destroy(tog_batch* b) {
    if (!b) return TOG_OK;
    if (b->own) cudaStreamSynchronize(b->own);
    if (b->stream && b->stream != b->own) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void* p : b->allocs) cudaFree(p);
    if (b->h_G) cudaFreeHost(b->h_G);
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return TOG_OK;
}

int tog_batch_set_stream(tog_batch* b, void* stream) {
    if (!b) return bfail(TOG_ERR_ARG, "null batch");
    TB_CUDA(cudaStreamSynchronize(b->stream));
    b->stream = stream ? (cudaStream_t)stream : b->own;
    return TOG_OK;
}

int tog_batch_step(tog_batch* b, tog_batch_stats* stats) {
    if (!b) return bfail(TOG_ERR_ARG, "null batch");
    TB_CUDA(cudaGraphLaunch(b->exec, b->stream));
    TB_CUDA(cudaMemcpyAsync(b->h_G, b->d_G, sizeof(BGlobal), cudaMemcpyDeviceToHost, b->stream));
    TB_CUDA(cudaStreamSynchronize(b->stream));
    ++b->steps;
    if (stats) {
        stats->pcg_loops = b->h_G->loops;
        stats->failed = b->h_G->failed;
        stats->steps = b->steps;
    }
    if (b->h_G->failed > 0)
        return bfail(TOG_NOT_CONVERGED, std::to_string(b->h_G->failed) + " problem(s) of the batch did not converge");
    return TOG_OK;
}

int tog_batch_results(tog_batch* b, double* compliance, double* change, int32_t* cg_iterations) {
    if (!b) return bfail(TOG_ERR_ARG, "null batch");
    TB_CUDA(cudaMemcpyAsync(b->h_B.data(), b->d_B, b->nprob * sizeof(BState), cudaMemcpyDeviceToHost, b->stream));
    TB_CUDA(cudaStreamSynchronize(b->stream));
    for (int p = 0; p < b->nprob; ++p) {
        if (compliance) compliance[p] = b->h_B[p].comp;
        if (change) change[p] = b->h_B[p].oc.change;
        if (cg_iterations) cg_iterations[p] = b->h_B[p].pcg.it;
    }
    return TOG_OK;
}

int tog_batch_get_design(tog_batch* b, int32_t prob, double* x) {
    if (!b || !x || prob < 0 || prob >= b->nprob) return bfail(TOG_ERR_ARG, "bad batch design request");
    const BProb& P = b->probs[prob];
    TB_CUDA(cudaMemcpyAsync(x, b->A.x + P.eoff, (size_t)P.nel[0] * P.nel[1] * sizeof(double), cudaMemcpyDeviceToHost,
                            b->stream));
    TB_CUDA(cudaStreamSynchronize(b->stream));
    return TOG_OK;
}

int tog_batch_autotune(tog_batch* b, int32_t* ly_out) {
    if (!b) return bfail(TOG_ERR_ARG, "null batch");
    // time the FP32 operator over all problems for each candidate chunk height and keep the fastest
    const int cand[] = {8, 16, 32, 64, 128};
    float best_ms = 1e30f;
    int best = b->LY;
    cudaEvent_t e0, e1;
    TB_CUDA(cudaEventCreate(&e0));
    TB_CUDA(cudaEventCreate(&e1));
    // operator inputs: every problem in PCG mode with beta = 0 (state only read by the operator)
    std::vector<BState> hb(b->nprob);
    TB_CUDA(cudaMemcpy(hb.data(), b->d_B, b->nprob * sizeof(BState), cudaMemcpyDeviceToHost));
    std::vector<BState> tb = hb;
    for (auto& s : tb) {
        s.mode = M_PCG;
        s.pcg.beta = 0.0;
    }
    for (int ly : cand) {
        build_mv_items(b, ly);
        TB_CUDA(cudaFree(b->d_mv));
        b->allocs.erase(std::remove(b->allocs.begin(), b->allocs.end(), (void*)b->d_mv), b->allocs.end());
        int rc = balloc(b, &b->d_mv, b->mv.size() + 4 * 64);
        if (rc != TOG_OK) return rc;
        TB_CUDA(cudaMemcpy(b->d_mv, b->mv.data(), b->mv.size() * sizeof(Item), cudaMemcpyHostToDevice));
        TB_CUDA(cudaMemcpy(b->d_P, b->probs.data(), b->nprob * sizeof(BProb), cudaMemcpyHostToDevice));
        BArgs A = b->A;
        A.mv = b->d_mv;
        A.nmv = (int)b->mv.size();
        A.LY = ly;
        const int nmvb = (A.nmv + kMvWarps - 1) / kMvWarps;
        for (int rep = 0; rep < 2; ++rep) {
            TB_CUDA(cudaMemcpy(b->d_B, tb.data(), b->nprob * sizeof(BState), cudaMemcpyHostToDevice));
            bk_matvec<float, MV_PCG><<<nmvb, 32 * kMvWarps, 0, b->own>>>(A);
        }
        TB_CUDA(cudaEventRecord(e0, b->own));
        for (int rep = 0; rep < 10; ++rep) bk_matvec<float, MV_PCG><<<nmvb, 32 * kMvWarps, 0, b->own>>>(A);
        TB_CUDA(cudaEventRecord(e1, b->own));
        TB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        TB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = ly;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    TB_CUDA(cudaMemcpy(b->d_B, hb.data(), b->nprob * sizeof(BState), cudaMemcpyHostToDevice));
    // rebuild items with the winner and re-record the graph
    build_mv_items(b, best);
    TB_CUDA(cudaFree(b->d_mv));
    b->allocs.erase(std::remove(b->allocs.begin(), b->allocs.end(), (void*)b->d_mv), b->allocs.end());
    int rc = balloc(b, &b->d_mv, b->mv.size() + 4 * 64);
    if (rc != TOG_OK) return rc;
    TB_CUDA(cudaMemcpy(b->d_mv, b->mv.data(), b->mv.size() * sizeof(Item), cudaMemcpyHostToDevice));
    TB_CUDA(cudaMemcpy(b->d_P, b->probs.data(), b->nprob * sizeof(BProb), cudaMemcpyHostToDevice));
    b->LY = best;
    b->A.mv = b->d_mv;
    b->A.nmv = (int)b->mv.size();
    b->A.LY = best;
    rc = build_graph(b);
    if (rc != TOG_OK) return rc;
    if (ly_out) *ly_out = best;
    return TOG_OK;
}

}  // extern "C"
