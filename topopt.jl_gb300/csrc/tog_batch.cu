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
constexpr int kOcMax = 100;        // bisection step cap
constexpr int kMaxLoops = 1 << 20; // PCG loop cap of one design iteration

enum { M_PCG = 0, M_RU = 1, M_DONE = 2, M_FAIL = 3, M_INIT = 4 };

struct BProb {
    int nel[2], nn[2];
    long long noff, eoff;        // first node / cell of the problem
    int t0, nt, ntx, pad;        // operator items (strip x band): first, count, strips along x
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
    int list_n[2], updates, pad; // listed problems per work list; reliable updates of the step
};

enum { kActive = 0, kRefresh = 1 };
constexpr int kListCache = 1024;   // work-list entries a block keeps in shared memory

struct WList {   // a work list (see the kernels' comments)
    int *prob, *tpref, *npref;
};

struct Item {   // one work item
    int prob;
    int a, b;   // matvec: x tile, y chunk start; node/cell items: chunk start
};

struct BArgs {
    const BProb* P;
    BState* B;
    BGlobal* G;
    const Item* nd;
    const Item* ce;
    int nnd, nce, nprob, LY;
    int in_graph;               // kernels set graph conditions only inside the graph
    int in_loop;                // ... and the refresh condition only inside the PCG loop body
    WList lst[2];
    const double* f;
    double *u, *r64;
    float *x32, *r32, *P0, *P1, *q32, *dinv32, *e32;
    double *e64, *vars, *x, *xnew, *dc, *dv, *grad, *B_oc, *nodal, *invW;
    const int* soff;
    const double* sw;
    double* partials;           // one slot per item (x2)
    Modal<float, 2> Mf;
    Modal<double, 2> Md;
    float Kc[2][4][2][4];       // element stiffness by [c][corner][d][corner] (FP32 gather operator)
    double xmin, pen, ru_delta2, move;
    int ip, maxit;
    cudaGraphConditionalHandle h_pcg, h_oc, h_ru;
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

__device__ int build_list(const BArgs& A, int l, int* failed);

// ---------------------------------------------------------------------------
// design iteration start: every problem to M_INIT, counters cleared, all listed
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
        A.G->updates = 0;
    }
    __syncthreads();
    build_list(A, kRefresh, nullptr);   // every problem starts with an FP64 residual
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
// Work lists.  The PCG-loop kernels run persistent grids that stride over the
// tiles (or node chunks) of listed problems only, so finished problems cost
// nothing in later loops:
//   list kActive:  problems in PCG mode (rebuilt after every refresh pass)
//   list kRefresh: problems needing the FP64 true residual (M_INIT or M_RU)
// List l holds, for its k-th problem (ascending ids): prob[k], the first tile of
// that problem in the flattened tile range (tpref[k], prefix sum, tpref[n] = total)
// and its first node chunk (npref[k]); n = G->list_n[l].  Blocks copy a list of up
// to CAP problems to shared memory and search it there.
__device__ __forceinline__ int ld_mode(const BState* B, int p) {
    return *(volatile const int*)&B[p].mode;
}

// block-wide exclusive scan of three counters; returns the block totals in tot[]
__device__ __forceinline__ void block_scan3(int (&v)[3], int (&tot)[3]) {
    __shared__ int sw[3][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int inc[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        inc[i] = v[i];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc[i], o);
            if (lane >= o) inc[i] += t;
        }
        if (lane == 31) sw[i][warp] = inc[i];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int x = lane < nw ? sw[i][lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += t;
            }
            sw[i][lane] = x;   // inclusive prefix of the warp totals
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int before = warp > 0 ? sw[i][warp - 1] : 0;
        tot[i] = sw[i][nw - 1];
        v[i] = before + inc[i] - v[i];
    }
    __syncthreads();
}

// Rebuild list l from the problem modes (all threads of ONE block, no other
// kernel running).  Returns the number listed; *failed (thread 0) = failed problems.
__device__ int build_list(const BArgs& A, int l, int* failed) {
    __shared__ int s_fail;
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();
    const WList& W = A.lst[l];
    int bk = 0, bt = 0, bn = 0, nf = 0;
    for (int b0 = 0; b0 < A.nprob; b0 += blockDim.x) {
        const int p = b0 + threadIdx.x;
        int v[3] = {0, 0, 0};
        if (p < A.nprob) {
            const int m = ld_mode(A.B, p);
            if (l == kActive ? (m == M_PCG) : (m == M_INIT || m == M_RU)) {
                v[0] = 1;
                v[1] = A.P[p].nt;
                v[2] = A.P[p].nnd;
            }
            nf += (m == M_FAIL);
        }
        const int flag = v[0];
        int tot[3];
        block_scan3(v, tot);
        if (flag) {
            W.prob[bk + v[0]] = p;
            W.tpref[bk + v[0]] = bt + v[1];
            W.npref[bk + v[0]] = bn + v[2];
        }
        bk += tot[0];
        bt += tot[1];
        bn += tot[2];
    }
    if (nf) atomicAdd(&s_fail, nf);
    __syncthreads();
    if (threadIdx.x == 0) {
        W.tpref[bk] = bt;
        W.npref[bk] = bn;
        A.G->list_n[l] = bk;
        __threadfence();
        if (failed) *failed = s_fail;
    }
    return bk;
}

struct ListView {
    const int* pref;
    const int* prob;
    int n, total;
};

template <bool TILES, int CAP>
__device__ __forceinline__ ListView load_list(const BArgs& A, int l, int* s_pref, int* s_prob) {
    const WList& W = A.lst[l];
    const int* gpref = TILES ? W.tpref : W.npref;
    ListView V;
    V.n = __ldcg(&A.G->list_n[l]);
    V.total = V.n > 0 ? __ldcg(gpref + V.n) : 0;
    V.pref = gpref;
    V.prob = W.prob;
    if (CAP > 0 && V.n > 0 && V.n <= CAP && V.total > (int)blockIdx.x) {
        for (int i = threadIdx.x; i <= V.n; i += blockDim.x) s_pref[i] = __ldcg(gpref + i);
        for (int i = threadIdx.x; i < V.n; i += blockDim.x) s_prob[i] = __ldcg(W.prob + i);
        __syncthreads();
        V.pref = s_pref;
        V.prob = s_prob;
    }
    return V;
}

// largest k in [0, n) with pref[k] <= w  (pref ascending, pref[0] = 0 <= w)
__device__ __forceinline__ int find_seg(const int* pref, int n, int w) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pref[mid] <= w)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Skip the rest of a listed problem ending at `end`: the loop increment then
// takes this block's stride past it.
__device__ __forceinline__ int skip_to(int w, int end) {
    const int G = gridDim.x;
    return w + ((end - w + G - 1) / G - 1) * G;
}

__device__ __forceinline__ void request_refresh(const BArgs& A) {
    if (A.in_loop) cudaGraphSetConditional(A.h_ru, 1u);
}

// ---------------------------------------------------------------------------
// Segmented reduction of the persistent loop kernels.  A block owns a
// contiguous range of work items (tiles or node chunks of the flattened list)
// and keeps its partial sums for one problem across consecutive items; at the
// end of the problem's items in its range it publishes them in the slot of the
// segment's first item (zeros in the other slots of the segment).  The block
// that completes a problem's item count sums the problem's slots in order, so
// the totals do not depend on timing.  Returns true in that block (tot[] set).
template <int NV>
__device__ bool seg_flush(double (&v)[NV], double* partials, int seg0, int wend, int pbeg, int pend,
                          unsigned* counter, double (&tot)[NV]) {
    __shared__ double sred[NV][32];
    __shared__ int amlast;
    block_reduce<NV, false>(v, sred);
    if (threadIdx.x < 32) {
        for (int i = seg0 + 1 + (int)threadIdx.x; i < wend; i += 32)
#pragma unroll
            for (int j = 0; j < NV; ++j) partials[(size_t)i * NV + j] = 0.0;
        if (threadIdx.x == 0)
#pragma unroll
            for (int j = 0; j < NV; ++j) partials[(size_t)seg0 * NV + j] = v[j];
        __threadfence();
        __syncwarp();
        if (threadIdx.x == 0) {
            const unsigned n = (unsigned)(wend - seg0);
            amlast = (atomicAdd(counter, n) + n == (unsigned)(pend - pbeg));
        }
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) s[j] = 0.0;
    for (int i = pbeg + (int)threadIdx.x; i < pend; i += blockDim.x)
#pragma unroll
        for (int j = 0; j < NV; ++j) s[j] += __ldcg(partials + (size_t)i * NV + j);
    block_reduce<NV, false>(s, sred);
#pragma unroll
    for (int j = 0; j < NV; ++j) tot[j] = s[j];
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// contiguous item range [w0, w1) of this block
__device__ __forceinline__ void block_range(int total, int& w0, int& w1) {
    w0 = (int)((long long)total * blockIdx.x / gridDim.x);
    w1 = (int)((long long)total * (blockIdx.x + 1) / gridDim.x);
}

// ---------------------------------------------------------------------------
// Matrix-free operator as a warp march.  A work item is a strip of 32 node
// columns (lanes; x = 30 cx - 1 + lane, lanes 1..30 own their column, lanes 0
// and 31 are halo) by a band of LY node rows of one problem.  The warp walks
// the node rows of the band (plus one above and one below); lane l applies the
// element to its upper right in modal form, its corner forces reach the nodes
// through warp shuffles (columns) and a register carry (rows).  The raw inputs
// of the next D rows are loaded ahead into a register ring, so each warp keeps
// D rows of loads in flight with no shared memory and no barriers.
//   MV_PCG (FP32):   p = D^-1 r + beta p_old, q = K p, p.q -> alpha   (list kActive)
//   MV_RESID (FP64): v = u + s x32 (fixed dofs zero), r64 = f - K v,
//                    ||r64||^2 -> refresh decision                   (list kRefresh)
// Warps own contiguous item ranges; partial sums are flushed per problem
// segment (slot of the segment's first item, zeros in the rest), and the warp
// completing a problem sums its slots in order.
template <int NV>
__device__ bool warp_seg_flush(double (&v)[NV], double* partials, int seg0, int wend, int pbeg, int pend,
                               unsigned* counter, double (&tot)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = warp_sum(v[j]);
    for (int i = seg0 + 1 + lane; i < wend; i += 32)
#pragma unroll
        for (int j = 0; j < NV; ++j) partials[(size_t)i * NV + j] = 0.0;
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) partials[(size_t)seg0 * NV + j] = v[j];
    __threadfence();
    __syncwarp();
    unsigned last = 0;
    if (lane == 0) {
        const unsigned n = (unsigned)(wend - seg0);
        last = (atomicAdd(counter, n) + n == (unsigned)(pend - pbeg)) ? 1u : 0u;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) s[j] = 0.0;
    for (int i = pbeg + lane; i < pend; i += 32)
#pragma unroll
        for (int j = 0; j < NV; ++j) s[j] += __ldcg(partials + (size_t)i * NV + j);
#pragma unroll
    for (int j = 0; j < NV; ++j) tot[j] = warp_sum(s[j]);
    if (lane == 0) *counter = 0u;
    return true;
}

#ifndef TOG_MARCH_DEPTH
#define TOG_MARCH_DEPTH 7
#endif
constexpr int kMarchDepth = TOG_MARCH_DEPTH;   // rows the FP32 operator loads ahead

template <typename T, int MODE>
struct MarchRow;
template <>
struct MarchRow<float, MV_PCG> {   // raw inputs of node row j and the density of element row j - 1
    float2 r, po;
    float d, rho;
};
template <>
struct MarchRow<double, MV_RESID> {   // ... and the load of node row j - 1
    double2 u, f;
    float2 xs;
    double rho;
};

constexpr int kMarchWarps = 8;   // warps per block
constexpr int kMarchList = 1024; // work-list entries a block keeps in shared memory

// The batch's problems are clamped along the left edge (x = 0) and nowhere else,
// so the fixed-dof mask of a node is a function of its column.

template <typename T, int MODE>
__global__ void __launch_bounds__(32 * kMarchWarps) bk_march(BArgs A) {
    constexpr int D = (MODE == MV_PCG) ? kMarchDepth : 2;   // rows loaded ahead (register ring)
    using Row = MarchRow<T, MODE>;
    using Acc = typename std::conditional<MODE == MV_PCG, float, double>::type;
    using V2 = typename std::conditional<MODE == MV_PCG, float2, double2>::type;
    __shared__ int s_pref[kMarchList + 1], s_prob[kMarchList];
    if (MODE == MV_PCG && blockIdx.x == 0 && threadIdx.x == 0) A.G->loops += 1;
    const ListView V = load_list<true, kMarchList>(A, MODE == MV_PCG ? kActive : kRefresh, s_pref, s_prob);
    const int lane = threadIdx.x & 31;
    const int GW = gridDim.x * kMarchWarps;
    const int gw = blockIdx.x * kMarchWarps + (threadIdx.x >> 5);
    const int w0 = (int)((long long)V.total * gw / GW), w1 = (int)((long long)V.total * (gw + 1) / GW);
    if (w0 >= w1) return;
    const Modal<T, 2>& M = *reinterpret_cast<const Modal<T, 2>*>(MODE == MV_PCG ? (const void*)&A.Mf : (const void*)&A.Md);
    const int LY = A.LY;
    int k = find_seg(V.pref, V.n, w0);
    int kbeg = V.pref[k], kend = V.pref[k + 1];
    int seg0 = w0;
    Acc acc = Acc(0);
    for (int w = w0; w < w1; ++w) {
        const int p = V.prob[k];
        const BProb& P = A.P[p];
        BState& S = A.B[p];
        const int nnx = P.nn[0], nny = P.nn[1], nelx = P.nel[0], nely = P.nel[1];
        const int t = w - kbeg;
        const int band = t / P.ntx, cx = t - band * P.ntx;
        const int b0 = band * LY, b1 = min(b0 + LY, nny);
        const int x = 30 * cx - 1 + lane;
        const bool colok = x >= 0 && x < nnx;
        const bool elok = x >= 0 && x < nelx && lane < 31;
        const bool own = colok && lane >= 1 && lane <= 30;
        const bool fixed = (x == 0);
        // 32-bit node / cell indices (the batch holds fewer than 2^30 nodes); used only where
        // the node or cell exists (x >= 0)
        const unsigned nb = (unsigned)P.noff + (unsigned)x, eb = (unsigned)P.eoff + (unsigned)x;
        // per-item scalars and row loader
        T beta = T(0), sc = T(0);
        int odd = 0, mode = 0;
        if (MODE == MV_PCG) {
            beta = (T)S.pcg.beta;
            odd = S.pcg.it & 1;
        } else {
            mode = S.mode;
            sc = (mode == M_RU) ? (T)S.s : T(0);
        }
        auto load = [&](int j, Row& R) {
            const bool rok = colok && j >= 0 && j < nny;
            const unsigned n = nb + (unsigned)nnx * (unsigned)j;
            const bool eok = elok && j >= 1 && j - 1 < nely;
            const unsigned e = eb + (unsigned)nelx * (unsigned)(j - 1);
            if constexpr (MODE == MV_PCG) {
                const float2* pold = reinterpret_cast<const float2*>(odd ? A.P0 : A.P1);
                R.r = rok ? reinterpret_cast<const float2*>(A.r32)[n] : make_float2(0.f, 0.f);
                R.po = rok ? pold[n] : make_float2(0.f, 0.f);
                R.d = rok ? A.dinv32[n] : 0.f;
                R.rho = eok ? A.e32[e] : 0.f;
            } else {
                R.u = rok ? reinterpret_cast<const double2*>(A.u)[n] : make_double2(0.0, 0.0);
                R.xs = rok ? reinterpret_cast<const float2*>(A.x32)[n] : make_float2(0.f, 0.f);
                R.rho = eok ? A.e64[e] : 0.0;
                R.f = (own && j >= 1) ? reinterpret_cast<const double2*>(A.f)[n - nnx] : make_double2(0.0, 0.0);
            }
        };
        const int j0 = b0 - 1, j1 = b1;   // node rows walked (inclusive)
        Row buf[D];
#pragma unroll
        for (int s = 0; s < D; ++s)
            if (j0 + s <= j1) load(j0 + s, buf[s]);
        V2 plo{}, plr{}, carry{};
        for (int jb = j0; jb <= j1; jb += D) {
#pragma unroll
            for (int s = 0; s < D; ++s) {
                const int j = jb + s;
                if (j > j1) break;
                const Row R = buf[s];
                if (j + D <= j1) load(j + D, buf[s]);
                V2 pj;
                if constexpr (MODE == MV_PCG) {
                    pj.x = fmaf(beta, R.po.x, R.d * M.kdinv[0] * R.r.x);
                    pj.y = fmaf(beta, R.po.y, R.d * M.kdinv[1] * R.r.y);
                } else {
                    pj.x = fixed ? 0.0 : fma(sc, (double)R.xs.x, R.u.x);
                    pj.y = fixed ? 0.0 : fma(sc, (double)R.xs.y, R.u.y);
                }
                V2 pr;
                pr.x = __shfl_down_sync(0xffffffffu, pj.x, 1);
                pr.y = __shfl_down_sync(0xffffffffu, pj.y, 1);
                if (j >= b0) {   // element row j - 1: corners (lo, lo right, up, up right)
                    T y[2][4] = {{plo.x, plr.x, pj.x, pr.x}, {plo.y, plr.y, pj.y, pr.y}};
                    element_apply<T, 2>(M, (T)R.rho, y);
                    const T t1x = __shfl_up_sync(0xffffffffu, y[0][1], 1);
                    const T t1y = __shfl_up_sync(0xffffffffu, y[1][1], 1);
                    const T t3x = __shfl_up_sync(0xffffffffu, y[0][3], 1);
                    const T t3y = __shfl_up_sync(0xffffffffu, y[1][3], 1);
                    if (j > b0 && own) {   // node row j - 1 is complete
                        const T qx = carry.x + y[0][0] + t1x, qy = carry.y + y[1][0] + t1y;
                        const unsigned n = nb + (unsigned)nnx * (unsigned)(j - 1);
                        if constexpr (MODE == MV_PCG) {
                            const float2 qv = fixed ? make_float2(0.f, 0.f) : make_float2(qx, qy);
                            reinterpret_cast<float2*>(odd ? A.P1 : A.P0)[n] = plo;
                            reinterpret_cast<float2*>(A.q32)[n] = qv;
                            acc = fmaf(plo.x, qv.x, fmaf(plo.y, qv.y, acc));
                        } else {
                            const double r0 = fixed ? 0.0 : R.f.x - qx;
                            const double r1 = fixed ? 0.0 : R.f.y - qy;
                            reinterpret_cast<double2*>(A.r64)[n] = make_double2(r0, r1);
                            acc = fma(r0, r0, fma(r1, r1, acc));
                        }
                    }
                    carry.x = y[0][2] + t3x;
                    carry.y = y[1][2] + t3y;
                }
                plo = pj;
                plr = pr;
            }
        }
        const bool last_of_prob = (w + 1 == kend);
        if (last_of_prob || w + 1 == w1) {
            double v[1] = {(double)acc}, tot[1];
            if (warp_seg_flush<1>(v, A.partials, seg0, w + 1, kbeg, kend, &S.cnt[MODE == MV_PCG ? 0 : 1], tot) &&
                lane == 0) {
                if (MODE == MV_PCG) {
                    S.pcg.pq = tot[0];
                    if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
                        S.mode = M_RU;   // breakdown: refresh from the true residual
                        request_refresh(A);
                    } else {
                        S.pcg.alpha = S.pcg.rz / tot[0];
                    }
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
            acc = Acc(0);
            seg0 = w + 1;
        }
        if (last_of_prob && w + 1 < w1) {
            ++k;
            kbeg = kend;
            kend = V.pref[k + 1];
        }
    }
}

// Reliable update / initialisation over the node chunks of listed problems in
// M_INIT or M_RU: u += s x32; then, unless converged, r32 = r64 / res, x32 = 0,
// the last direction rescaled (M_RU) or cleared (M_INIT), and the PCG scalars
// rebuilt.  The last block of the grid rebuilds the active list and sets the
// PCG-loop condition.
__global__ void __launch_bounds__(kBThreads) bk_rescale(BArgs A) {
    __shared__ int s_pref[kListCache + 1], s_prob[kListCache];
    const ListView V = load_list<false, kListCache>(A, kRefresh, s_pref, s_prob);
    for (int w = blockIdx.x; w < V.total; w += gridDim.x) {
        const int k = find_seg(V.pref, V.n, w);
        const int p = V.prob[k];
        BState& S = A.B[p];
        const int mode = S.mode;
        if (mode != M_INIT && mode != M_RU) {   // converged from the start (M_DONE) or failed
            w = skip_to(w, V.pref[k + 1]);
            continue;
        }
        const BProb& P = A.P[p];
        const int c = w - V.pref[k];
        const bool conv = S.stall == -1;
        const long long nnodes = (long long)P.nn[0] * P.nn[1];
        const double s_old = (mode == M_RU) ? S.s : 0.0;
        const double res = S.res;
        const double inv = res > 0.0 ? 1.0 / res : 0.0;
        const int itn = S.pcg.it;
        float* plast = ((itn - 1) & 1) ? A.P1 : A.P0;
        const float ratio = (float)(res > 0.0 ? s_old / res : 0.0);
        float arz = 0.f, arr = 0.f;
        for (int tt = threadIdx.x; tt < kNodeChunk; tt += blockDim.x) {
            const long long nl = (long long)c * kNodeChunk + tt;
            if (nl >= nnodes) break;
            const long long n = P.noff + nl;
            const float d = A.dinv32[n];
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const long long i = 2 * n + cc;
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
                    arz = fmaf(rn, d * A.Mf.kdinv[cc] * rn, arz);
                    arr = fmaf(rn, rn, arr);
                }
            }
        }
        double v[2] = {arz, arr}, tot[2];
        if (prob_reduce_block<2>(v, A.partials, P.nd0 + c, P.nd0, P.nnd, &S.cnt[2], tot)) {
            if (threadIdx.x == 0) {
                if (conv) {
                    S.mode = M_DONE;
                } else {
                    if (mode == M_RU) {
                        const double q = s_old / res;
                        const double rz_prev = S.pcg.rz_old * q * q;
                        S.pcg.beta = rz_prev > 0.0 ? tot[0] / rz_prev : 0.0;
                        S.updates += 1;
                        atomicAdd(&A.G->updates, 1);
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
        __syncthreads();
    }
    if (grid_last(&A.G->cnt[0])) {
        int failed = 0;
        const int active = build_list(A, kActive, &failed);
        if (threadIdx.x == 0) {
            A.G->active = active;
            A.G->failed = failed;
            if (A.in_graph) cudaGraphSetConditional(A.h_pcg, (active > 0 && A.G->loops < kMaxLoops) ? 1u : 0u);
            if (A.in_loop) cudaGraphSetConditional(A.h_ru, 0u);
        }
    }
}

// PCG update over the node chunks of listed problems in M_PCG:
// x += alpha p, r -= alpha q, r.z, r.r
__global__ void __launch_bounds__(kBThreads) bk_update(BArgs A) {
    __shared__ int s_pref[kListCache + 1], s_prob[kListCache];
    const ListView V = load_list<false, kListCache>(A, kActive, s_pref, s_prob);
    int w, w1;
    block_range(V.total, w, w1);
    const float k0 = A.Mf.kdinv[0], k1 = A.Mf.kdinv[1];
    const float2* __restrict__ qq = reinterpret_cast<const float2*>(A.q32);
    float2* __restrict__ xx = reinterpret_cast<float2*>(A.x32);
    float2* __restrict__ rr = reinterpret_cast<float2*>(A.r32);
    while (w < w1) {
        const int k = find_seg(V.pref, V.n, w);
        const int kbeg = V.pref[k], kend = V.pref[k + 1];
        const int wend = min(kend, w1);
        const int p = V.prob[k];
        BState& S = A.B[p];
        if (S.mode != M_PCG) {   // broke down in the operator pass
            w = wend;
            continue;
        }
        const BProb& P = A.P[p];
        const int itn = S.pcg.it;
        const float2* __restrict__ pp = reinterpret_cast<const float2*>((itn & 1) ? A.P1 : A.P0);
        const float alpha = (float)S.pcg.alpha;
        const long long nnodes = (long long)P.nn[0] * P.nn[1];
        const long long nb = (long long)(w - kbeg) * kNodeChunk;
        const long long ne = min(nnodes, (long long)(wend - kbeg) * kNodeChunk);
        float arz = 0.f, arr = 0.f;
        for (long long base = nb; base < ne; base += 4 * kBThreads) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const long long nl = base + u * kBThreads + threadIdx.x;
                if (nl < ne) {
                    const long long n = P.noff + nl;
                    const float d = A.dinv32[n];
                    const float2 pv = pp[n], qv = qq[n];
                    float2 xv = xx[n], rv = rr[n];
                    xv.x = fmaf(alpha, pv.x, xv.x);
                    xv.y = fmaf(alpha, pv.y, xv.y);
                    rv.x = fmaf(-alpha, qv.x, rv.x);
                    rv.y = fmaf(-alpha, qv.y, rv.y);
                    xx[n] = xv;
                    rr[n] = rv;
                    arz = fmaf(rv.x, d * k0 * rv.x, arz);
                    arz = fmaf(rv.y, d * k1 * rv.y, arz);
                    arr = fmaf(rv.x, rv.x, arr);
                    arr = fmaf(rv.y, rv.y, arr);
                }
            }
        }
        double v[2] = {arz, arr}, tot[2];
        if (seg_flush<2>(v, A.partials, w, wend, kbeg, kend, &S.cnt[3], tot) && threadIdx.x == 0) {
            PcgState& st = S.pcg;
            const double rzo = st.rz;
            st.rz_old = rzo;
            st.rz = tot[0];
            st.beta = rzo != 0.0 ? tot[0] / rzo : 0.0;
            st.rr = tot[1];
            st.it = itn + 1;
            if (!isfinite(tot[1]) || tot[1] <= st.tol2 || tot[1] < st.ru_delta2 * st.rr_max ||
                itn + 1 >= st.maxit) {   // at maxit the refresh pass decides (and fails the problem)
                S.mode = M_RU;
                request_refresh(A);
            }
            st.rr_max = fmax(st.rr_max, tot[1]);
        }
        __syncthreads();
        w = wend;
    }
}


// refresh list of the problems that asked for the FP64 residual in this loop
__global__ void bk_rulist(BArgs A) { build_list(A, kRefresh, nullptr); }

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
        __shared__ int s_act;
        if (threadIdx.x == 0) s_act = 0;
        __syncthreads();
        int act = 0;
        for (int b = threadIdx.x; b < A.nprob; b += blockDim.x) act += !*(volatile const int*)&A.B[b].oc.done;
        if (act) atomicAdd(&s_act, act);
        __syncthreads();
        if (threadIdx.x == 0) {
            A.G->oc_active = s_act;
            if (A.in_graph) cudaGraphSetConditional(A.h_oc, s_act > 0 ? 1u : 0u);
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
    std::vector<Item> nd, ce;
    long long nnodes = 0, ncells = 0;
    int LY = 32;                 // node rows per operator item (autotuned)
    int gt = 0, gr = 0, gn = 0;  // persistent grids: FP32 operator, FP64 residual, node passes
    int grid_div = 1;            // FP32 operator grid = occupancy limit / grid_div (autotuned)
    double xmin = 1e-9, pen = 3.0, rtol = 1e-8, move = 0.2;
    int maxit = 1 << 20;
    cudaStream_t own = nullptr, stream = nullptr;
    int nsm = 152;
    // device
    BProb* d_P = nullptr;
    BState* d_B = nullptr;
    BGlobal* d_G = nullptr;
    Item *d_nd = nullptr, *d_ce = nullptr;
    std::vector<void*> allocs;
    BArgs A{};
    std::vector<BState> h_B;
    BGlobal* h_G = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle h_pcg{}, h_oc{}, h_ru{};
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

// march items per problem: strips of 30 owned node columns x bands of LY node
// rows; returns the total
long long build_tiles(tog_batch* b, int LY) {
    long long t = 0;
    for (int p = 0; p < b->nprob; ++p) {
        BProb& P = b->probs[p];
        P.ntx = (P.nn[0] + 29) / 30;
        P.t0 = (int)t;
        P.nt = P.ntx * ((P.nn[1] + LY - 1) / LY);
        t += P.nt;
    }
    return t;
}

int blocks_per_sm(const void* fn, int threads, size_t smem = 0) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess || nb < 1) nb = 1;
    return nb;
}

void launch_mvpcg(const BArgs& A, int grid, cudaStream_t s) {
    bk_march<float, MV_PCG><<<grid, 32 * kMarchWarps, 0, s>>>(A);
}
void launch_resid(const BArgs& A, int grid, cudaStream_t s) {
    bk_march<double, MV_RESID><<<grid, 32 * kMarchWarps, 0, s>>>(A);
}

// persistent grid sizes; frac_div divides the FP32 operator's grid
void set_grids(tog_batch* b, int frac_div) {
    b->gt = std::max(1, b->nsm * blocks_per_sm((const void*)bk_march<float, MV_PCG>, 32 * kMarchWarps) / frac_div);
    b->gr = b->nsm * blocks_per_sm((const void*)bk_march<double, MV_RESID>, 32 * kMarchWarps);
    b->gn = b->nsm * blocks_per_sm((const void*)bk_update, kBThreads);
}

// design-iteration set-up: filter, element scales, Jacobi diagonal, FP64
// residual of the warm start, PCG initialisation (and the first active list)
void launch_setup(tog_batch* b, const BArgs& A, cudaStream_t s) {
    bk_begin<<<1, 256, 0, s>>>(A);
    bk_filt_nodeavg<<<A.nnd, kBThreads, 0, s>>>(A, A.x, A.nodal);
    bk_filt_cone<<<A.nce, kBThreads, 0, s>>>(A, A.nodal, A.x, A.vars);
    bk_escale<<<A.nce, kBThreads, 0, s>>>(A);
    bk_nodesum<<<A.nnd, kBThreads, 0, s>>>(A);
    launch_resid(A, b->gr, s);
    bk_rescale<<<b->gn, kBThreads, 0, s>>>(A);
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
    b->A.in_graph = 1;
    b->A.in_loop = 0;
    b->A.LY = b->LY;
    const BArgs A = b->A;
    cudaStream_t s = b->own;
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
    launch_setup(b, A, s);
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
    // body: FP32 operator + update every loop; the FP64 refresh pass (refresh list,
    // true residual, rescale) only in loops where some problem asked for it
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    TB_CUDA(cudaGraphConditionalHandleCreate(&b->h_ru, body, 0, cudaGraphCondAssignDefault));
    BArgs AL = A;
    AL.in_loop = 1;
    AL.h_ru = b->h_ru;
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    launch_mvpcg(AL, b->gt, s);
    bk_update<<<b->gn, kBThreads, 0, s>>>(AL);
    {
        int rc = tail(deps);
        if (rc != TOG_OK) return rc;
    }
    cudaGraph_t gb;
    TB_CUDA(cudaStreamEndCapture(s, &gb));
    cudaGraphNodeParams ci{};
    ci.type = cudaGraphNodeTypeConditional;
    ci.conditional.handle = b->h_ru;
    ci.conditional.type = cudaGraphCondTypeIf;
    ci.conditional.size = 1;
    cudaGraphNode_t nif;
    TB_CUDA(cudaGraphAddNode(&nif, body, deps.data(), nullptr, deps.size(), &ci));
    cudaGraph_t ibody = ci.conditional.phGraph_out[0];
    TB_CUDA(cudaStreamBeginCaptureToGraph(s, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    bk_rulist<<<1, 256, 0, s>>>(AL);
    launch_resid(AL, b->gr, s);
    bk_rescale<<<b->gn, kBThreads, 0, s>>>(AL);
    cudaGraph_t gib;
    TB_CUDA(cudaStreamEndCapture(s, &gib));
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
    // corner-ordered element block for the FP32 gather: corner n = bx + 2 by holds
    // Ferrite node a with kFerriteToCorner[a] = n, whose dofs are 2 a + c in Ke
    float Kc[2][4][2][4];
    {
        int c2f[4];
        for (int a = 0; a < 4; ++a) c2f[kFerriteToCorner[a]] = a;
        for (int c = 0; c < 2; ++c)
            for (int i = 0; i < 4; ++i)
                for (int d = 0; d < 2; ++d)
                    for (int j = 0; j < 4; ++j) Kc[c][i][d][j] = (float)Ke[(2 * c2f[i] + c) * 8 + 2 * c2f[j] + d];
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
    if (noff >= (1LL << 30)) {   // the operator kernels index nodes and dofs in 32 bits
        delete b;
        return bfail(TOG_ERR_ARG, "tog_batch_create: the batch needs fewer than 2^30 nodes in all");
    }
    const long long max_tiles = build_tiles(b, 8);   // the lowest band gives the most items
    build_tiles(b, b->LY);
    if (max_tiles > (1LL << 30)) {
        delete b;
        return bfail(TOG_ERR_ARG, "tog_batch_create: batch too large");
    }
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
    double* f = nullptr;
    int* d_soff = nullptr;
    double* d_sw = nullptr;
    R(balloc(b, &b->d_P, nprob));
    R(balloc(b, &b->d_B, nprob));
    R(balloc(b, &b->d_G, 1));
    for (int l = 0; l < 2; ++l) {
        R(balloc(b, &A.lst[l].prob, nprob + 1));
        R(balloc(b, &A.lst[l].tpref, nprob + 1));
        R(balloc(b, &A.lst[l].npref, nprob + 1));
    }
    R(balloc(b, &b->d_nd, b->nd.size()));
    R(balloc(b, &b->d_ce, b->ce.size()));
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
    const size_t nitems = std::max((size_t)max_tiles, std::max(b->nd.size(), b->ce.size()));
    R(balloc(b, &A.partials, 2 * nitems + 64));
    if (rc != TOG_OK) {
        std::string m = tog_last_error();
        tog_batch_destroy(b);
        bfail(rc, m);
        return rc;
    }
    // loads: unit load [0, -1] at node (nelx, load_j); the clamped left edge is
    // applied by the operator kernel (nodes of column 0)
    std::vector<double> hf(2 * NN, 0.0);
    for (int p = 0; p < nprob; ++p) {
        const BProb& P = b->probs[p];
        hf[2 * (P.noff + P.nel[0] + (long long)P.nn[0] * load_j[p]) + 1] = -1.0;
    }
    A.P = b->d_P;
    A.B = b->d_B;
    A.G = b->d_G;
    A.nd = b->d_nd;
    A.ce = b->d_ce;
    A.nnd = (int)b->nd.size();
    A.nce = (int)b->ce.size();
    A.nprob = nprob;
    A.LY = b->LY;
    std::memcpy(A.Kc, Kc, sizeof(Kc));
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
    C(cudaMemcpyAsync(b->d_nd, b->nd.data(), b->nd.size() * sizeof(Item), cudaMemcpyHostToDevice, b->own));
    C(cudaMemcpyAsync(b->d_ce, b->ce.data(), b->ce.size() * sizeof(Item), cudaMemcpyHostToDevice, b->own));
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
    set_grids(b, b->grid_div);
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
        stats->reliable_updates = b->h_G->updates;
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

int tog_batch_solve_info(tog_batch* b, double* residual, int32_t* refreshes, int32_t* status) {
    if (!b) return bfail(TOG_ERR_ARG, "null batch");
    TB_CUDA(cudaMemcpyAsync(b->h_B.data(), b->d_B, b->nprob * sizeof(BState), cudaMemcpyDeviceToHost, b->stream));
    TB_CUDA(cudaStreamSynchronize(b->stream));
    for (int p = 0; p < b->nprob; ++p) {
        const BState& S = b->h_B[p];
        if (residual) residual[p] = S.res;
        if (refreshes) refreshes[p] = S.updates;
        if (status) status[p] = S.mode == M_DONE ? TOG_OK : S.mode == M_FAIL ? TOG_NOT_CONVERGED : TOG_ERR_STATE;
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

int tog_batch_set_tile_rows(tog_batch* b, int32_t tile_rows) {
    if (!b || (tile_rows != 8 && tile_rows != 16 && tile_rows != 32 && tile_rows != 64))
        return bfail(TOG_ERR_ARG, "tog_batch_set_tile_rows: rows must be 8, 16, 32 or 64");
    TB_CUDA(cudaStreamSynchronize(b->stream));
    b->LY = tile_rows;
    b->grid_div = 1;
    build_tiles(b, tile_rows);
    TB_CUDA(cudaMemcpy(b->d_P, b->probs.data(), b->nprob * sizeof(BProb), cudaMemcpyHostToDevice));
    set_grids(b, 1);
    b->A.LY = tile_rows;
    return build_graph(b);
}

int tog_batch_autotune(tog_batch* b, int32_t* tile_rows) {
    if (!b) return bfail(TOG_ERR_ARG, "null batch");
    TB_CUDA(cudaStreamSynchronize(b->stream));
    // Every candidate (tile rows x grid size of the FP32 operator) is timed on
    // PCG iterations of all problems at once.  The PCG state comes from the
    // set-up kernels of a design iteration run outside the graph, with reliable
    // updates switched off so that every problem keeps iterating; only scratch
    // vectors change (the next design iteration rebuilds them).
    cudaStream_t s = b->own;
    const int cand_ty[] = {8, 16, 32, 64};
    const int cand_div[] = {1, 2, 4};
    float best_ms = 1e30f;
    int best_ty = b->LY, best_div = b->grid_div;
    cudaEvent_t e0, e1;
    TB_CUDA(cudaEventCreate(&e0));
    TB_CUDA(cudaEventCreate(&e1));
    int rc = TOG_OK;
    for (int ty : cand_ty) {
        build_tiles(b, ty);
        TB_CUDA(cudaMemcpyAsync(b->d_P, b->probs.data(), b->nprob * sizeof(BProb), cudaMemcpyHostToDevice, s));
        b->LY = ty;
        set_grids(b, 1);
        BArgs A = b->A;
        A.in_graph = 0;
        A.ru_delta2 = 0.0;
        A.LY = ty;
        launch_setup(b, A, s);
        for (int div : cand_div) {
            set_grids(b, div);
            for (int rep = 0; rep < 3; ++rep) {
                launch_mvpcg(A, b->gt, s);
                bk_update<<<b->gn, kBThreads, 0, s>>>(A);
            }
            TB_CUDA(cudaEventRecord(e0, s));
            for (int rep = 0; rep < 10; ++rep) {
                launch_mvpcg(A, b->gt, s);
                bk_update<<<b->gn, kBThreads, 0, s>>>(A);
            }
            TB_CUDA(cudaEventRecord(e1, s));
            TB_CUDA(cudaEventSynchronize(e1));
            TB_CUDA(cudaGetLastError());
            float ms = 0.f;
            TB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best_ms) {
                best_ms = ms;
                best_ty = ty;
                best_div = div;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->LY = best_ty;
    b->grid_div = best_div;
    build_tiles(b, best_ty);
    TB_CUDA(cudaMemcpyAsync(b->d_P, b->probs.data(), b->nprob * sizeof(BProb), cudaMemcpyHostToDevice, s));
    TB_CUDA(cudaStreamSynchronize(s));
    set_grids(b, best_div);
    b->A.LY = best_ty;
    rc = build_graph(b);
    if (rc != TOG_OK) return rc;
    if (tile_rows) *tile_rows = best_ty;
    return TOG_OK;
}

// Measurement hooks.  Launch one loop kernel nlaunch times over ALL problems of
// the batch on the batch's stream and return the mean time per launch (CUDA
// events).  State: the set-up kernels of a design iteration run first, outside
// the graph (reliable updates off, so every problem stays in PCG mode); only
// solver scratch changes, the design and displacements do not.
//   kernel 0: FP32 operator (p update, K p, p.q)    1: PCG vector update
//   kernel 2: FP64 true residual                      3: operator + update (one loop)
int tog_batch_bench_kernel(tog_batch* b, int32_t kernel, int32_t nlaunch, double* us_per_launch) {
    if (!b || kernel < 0 || kernel > 3 || nlaunch < 1 || !us_per_launch)
        return bfail(TOG_ERR_ARG, "tog_batch_bench_kernel: bad arguments");
    TB_CUDA(cudaStreamSynchronize(b->stream));
    cudaStream_t s = b->own;
    BArgs A = b->A;
    A.in_graph = 0;
    A.in_loop = 0;
    A.ru_delta2 = 0.0;
    launch_setup(b, A, s);
    if (kernel == 2) bk_begin<<<1, 256, 0, s>>>(A);   // every problem listed for the residual, mode M_INIT
    auto one = [&]() {
        if (kernel == 0 || kernel == 3) launch_mvpcg(A, b->gt, s);
        if (kernel == 1 || kernel == 3) bk_update<<<b->gn, kBThreads, 0, s>>>(A);
        if (kernel == 2) launch_resid(A, b->gr, s);
    };
    for (int i = 0; i < 3; ++i) one();
    cudaEvent_t e0, e1;
    TB_CUDA(cudaEventCreate(&e0));
    TB_CUDA(cudaEventCreate(&e1));
    TB_CUDA(cudaEventRecord(e0, s));
    for (int i = 0; i < nlaunch; ++i) one();
    TB_CUDA(cudaEventRecord(e1, s));
    TB_CUDA(cudaEventSynchronize(e1));
    TB_CUDA(cudaGetLastError());
    float ms = 0.f;
    TB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *us_per_launch = 1e3 * (double)ms / nlaunch;
    return TOG_OK;
}

// Algorithmic HBM bytes of one launch of those kernels over all problems: each
// array element read or written once (halo re-reads and scalars excluded).
int tog_batch_kernel_bytes(tog_batch* b, int32_t kernel, double* bytes) {
    if (!b || kernel < 0 || kernel > 3 || !bytes) return bfail(TOG_ERR_ARG, "tog_batch_kernel_bytes: bad arguments");
    const double N = (double)b->nnodes, C = (double)b->ncells;
    // operator: r32, p_old (8+8), dinv (4), fixed mask (1) in; p, q (8+8) out; densities (4 per cell)
    const double op = 37.0 * N + 4.0 * C;
    // update: p, q, x, r (4 x 8), dinv (4) in; x, r (2 x 8) out
    const double up = 52.0 * N;
    // residual: u (16), x32 (8), mask (1), f (16) in; r64 (16) out; densities (8 per cell)
    const double rs = 57.0 * N + 8.0 * C;
    *bytes = kernel == 0 ? op : kernel == 1 ? up : kernel == 2 ? rs : op + up;
    return TOG_OK;
}

}  // extern "C"
