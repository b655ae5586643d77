// 3D hex8 matrix-free operator without redundant work (sm_103a).
//
// Tiling.  A block owns a tile of 32 (x) x MV3_BY (y) element columns and a
// chunk of LZ element layers, marching in z; every element is evaluated by
// exactly one thread.  A node is *owned* by the tile of the element whose lower
// corner it is (clamped at the upper domain faces).  The owner writes its partial
// sum to q; a tile that touches a node on its upper x / y / z face, whose owner
// is the neighbouring tile, writes its partial to one of seven small side
// buffers (class x, y, z, xy, xz, yz, xyz).  The consumer (the PCG update or the
// finalize kernel) adds the side partials back in a fixed order, so the result
// is deterministic and no atomics are used.  The p.q partial sums of the fused
// PCG mode are taken over every emitted partial, which adds up to p.q by
// linearity.
//
// Inside a block: node contributions combine across x by warp shuffles, across
// y through shared memory and across z in registers.  Each thread computes the
// operator's input (the PCG direction p = D^-1 r + beta p_old, or the masked x)
// only at its own node; neighbours' values arrive by shuffle (x) and shared
// memory (y), and the loads of the plane two layers ahead are issued one layer
// early to hide the HBM latency.
#pragma once
#include "tog_kernels.cuh"

namespace tog {

constexpr int MV3_BY = 8;   // warps per block = element rows per tile

// n / d for n < 2^31 by multiply-shift (Granlund-Montgomery, m = ceil(2^(32+s) / d)).
struct FastDiv {
    unsigned long long m;
    unsigned s;
    unsigned d;
};
inline FastDiv make_fastdiv(unsigned d) {
    unsigned s = 0;
    while ((1ull << s) < d) ++s;
    FastDiv f;
    f.m = (((1ull << (32 + s)) + d - 1) / d);
    f.s = 32 + s;
    f.d = d;
    return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv& f) {
    return (unsigned)(((unsigned long long)n * f.m) >> f.s);
}

template <typename T>
struct Mv3Args {
    // operator input / output
    const T* x;            // PLAIN / RESID input (internal layout)
    const T* r;            // PCG residual
    T* P0;                 // PCG directions (ping-pong by iteration parity)
    T* P1;
    T* q;                  // owner partials (complete for interior nodes)
    T* side[8];            // side partials by class (index 1..7; 0 unused)
    const T* escale;       // per element E_e
    const T* dinv;         // per node 1 / sum_e E_e
    const uint8_t* fixmask;
    int nel[3];
    int nn[3];
    int nt[3];             // tiles in x, y, z
    int LZ;                // layers per z chunk
    FastDiv div_nnx, div_nny, div_nnz;
    PcgState* st;
    double* partials;
    Modal<T, 3> M;
};

// Index of node (i, j, k) in the side buffer of class cls (bit 0 = x, 1 = y, 2 = z).
template <typename T>
__device__ __forceinline__ long long side_index(const Mv3Args<T>& A, int cls, int i, int j, int k) {
    const int mx = i >> 5, my = j / MV3_BY, mz = k / A.LZ;
    const long long nnx = A.nn[0], nny = A.nn[1], nnz = A.nn[2];
    const long long tx = A.nt[0] - 1, ty = A.nt[1] - 1, tz = A.nt[2] - 1;
    switch (cls) {
        case 1: return ((long long)(mx - 1) * nnz + k) * nny + j;
        case 2: return ((long long)(my - 1) * nnz + k) * nnx + i;
        case 4: return ((long long)(mz - 1) * nny + j) * nnx + i;
        case 3: return ((long long)(mx - 1) * ty + (my - 1)) * nnz + k;
        case 5: return ((long long)(mx - 1) * tz + (mz - 1)) * nny + j;
        case 6: return ((long long)(my - 1) * tz + (mz - 1)) * nnx + i;
        default: return ((long long)(mx - 1) * ty + (my - 1)) * tz + (mz - 1);
    }
}

// Element count of each side class.
inline long long side_count(int cls, const int nn[3], const int nt[3]) {
    const long long tx = nt[0] - 1, ty = nt[1] - 1, tz = nt[2] - 1;
    switch (cls) {
        case 1: return tx * nn[2] * nn[1];
        case 2: return ty * nn[2] * nn[0];
        case 4: return tz * nn[1] * nn[0];
        case 3: return tx * ty * nn[2];
        case 5: return tx * tz * nn[1];
        case 6: return ty * tz * nn[0];
        default: return tx * ty * tz;
    }
}

// q_final at node (i, j, k): the owner partial plus the side partials of the
// tiles below it in x, y and z (fixed order).
template <typename T>
__device__ __forceinline__ void gather_q(const Mv3Args<T>& A, long long n, int i, int j, int k, T (&v)[3]) {
    const bool fx = (i & 31) == 0 && i > 0 && i < A.nel[0];
    const bool fy = (j % MV3_BY) == 0 && j > 0 && j < A.nel[1];
    const bool fz = (k % A.LZ) == 0 && k > 0 && k < A.nel[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = A.q[3 * n + c];
    if (fx | fy | fz) {
#pragma unroll
        for (int cls = 1; cls < 8; ++cls) {
            const bool on = ((cls & 1) ? fx : true) && ((cls & 2) ? fy : true) && ((cls & 4) ? fz : true);
            if (on) {
                const long long s = side_index(A, cls, i, j, k);
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] += A.side[cls][3 * s + c];
            }
        }
    }
}

template <typename T, int MODE>
__device__ __forceinline__ void mv3_emit(const Mv3Args<T>& A, T* __restrict__ pnew, int cls, int i, int j, int k,
                                         const T (&v)[3], const T (&pv)[3], T& dot) {
    if (cls == 0) {
        const long long n = i + (long long)A.nn[0] * (j + (long long)A.nn[1] * k);
#pragma unroll
        for (int c = 0; c < 3; ++c) A.q[3 * n + c] = v[c];
        if (MODE == MV_PCG) {
#pragma unroll
            for (int c = 0; c < 3; ++c) pnew[3 * n + c] = pv[c];
        }
    } else {
        const long long s = side_index(A, cls, i, j, k);
#pragma unroll
        for (int c = 0; c < 3; ++c) A.side[cls][3 * s + c] = v[c];
    }
    if (MODE == MV_PCG) {
#pragma unroll
        for (int c = 0; c < 3; ++c) dot = fma(pv[c], v[c], dot);
    }
}

// Raw loads for the operator input at one node (issued early, consumed later).
template <typename T, int MODE>
struct NodeRaw {
    T a[3];   // r (PCG) or x (PLAIN / RESID)
    T b[3];   // p_old (PCG)
    T d;      // D^-1 (PCG)
    unsigned m;
};

template <typename T, int MODE>
__device__ __forceinline__ void node_load(const Mv3Args<T>& A, const T* __restrict__ pold, int i, int j, int k,
                                          bool ok, NodeRaw<T, MODE>& R) {
    if (ok) {
        const long long n = i + (long long)A.nn[0] * (j + (long long)A.nn[1] * k);
        if (MODE == MV_PCG) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                R.a[c] = A.r[3 * n + c];
                R.b[c] = pold[3 * n + c];
            }
            R.d = A.dinv[n];
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) R.a[c] = A.x[3 * n + c];
            R.m = A.fixmask[n];
        }
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) R.a[c] = R.b[c] = T(0);
        R.d = T(0);
        R.m = 7u;
    }
}

template <typename T, int MODE>
__device__ __forceinline__ void node_value(const Mv3Args<T>& A, T beta, const NodeRaw<T, MODE>& R, T (&v)[3]) {
    if (MODE == MV_PCG) {
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = fma(beta, R.b[c], R.d * A.M.kdinv[c] * R.a[c]);
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = ((R.m >> c) & 1u) ? T(0) : R.a[c];
    }
}

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int MV3_STAGES = 3;   // raw-input ring: planes k+2 and k+3 in flight

// Raw PCG inputs of one node (r[3], p_old[3], D^-1), copied asynchronously.
template <typename T>
struct Mv3Ring {
    T own[MV3_STAGES][MV3_BY][32][7];
    T rgt[MV3_STAGES][MV3_BY][7];
    T top[MV3_STAGES][32][7];
    T cor[MV3_STAGES][7];
};

template <typename T>
struct Mv3Smem {
    T row[2][MV3_BY][32][2][3];   // output rows ey+1 (bz, c), by layer parity
    T rrow[2][MV3_BY][2][3];      // lane 31's right-column row ey+1
    T in[2][MV3_BY][32][2][3];    // operator input of a plane: own node, right neighbour
    Mv3Ring<T> ring;               // PCG mode: asynchronous copies of the next planes' raw inputs
};

template <typename T, int MODE>
__global__ void __launch_bounds__(32 * MV3_BY, sizeof(T) == 4 ? 3 : 1) k_mv3(const Mv3Args<T> A) {
    constexpr int BY = MV3_BY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Mv3Smem<T>& S = *reinterpret_cast<Mv3Smem<T>*>(smem_raw);
    const int lane = threadIdx.x, w = threadIdx.y;
    T beta = T(0);
    const T* __restrict__ pold = nullptr;
    T* __restrict__ pnew = nullptr;
    if (MODE == MV_PCG) {
        if (A.st->done) return;
        const int it = A.st->it;
        pnew = (it & 1) ? A.P1 : A.P0;
        pold = (it & 1) ? A.P0 : A.P1;
        beta = (T)A.st->beta;
    }
    const int nelx = A.nel[0], nely = A.nel[1], nelz = A.nel[2];
    const int ex = 32 * (int)blockIdx.x + lane;
    const int ey = BY * (int)blockIdx.y + w;
    const int kz0 = A.LZ * (int)blockIdx.z;
    const int kz1 = min(kz0 + A.LZ, nelz);
    const bool elxy = ex < nelx && ey < nely;
    const bool own_xy = ex <= nelx && ey <= nely;
    const bool last_lane = lane == 31, last_warp = w == BY - 1;
    const bool has_r = last_lane && ex + 1 <= nelx && ey <= nely;
    const bool has_t = last_warp && ey + 1 <= nely && ex <= nelx;
    const bool has_c = last_lane && last_warp && ex + 1 <= nelx && ey + 1 <= nely;
    const int clsx = (ex + 1 < nelx) ? 1 : 0;
    const int clsy = (ey + 1 < nely) ? 2 : 0;

    // operator input at this thread's node(s) of plane kk
    auto plane_inputs = [&](int kk, T (&own)[3], T (&rgt)[3], T (&top)[3], T (&cor)[3]) {
        NodeRaw<T, MODE> R;
        node_load<T, MODE>(A, pold, ex, ey, kk, own_xy, R);
        node_value<T, MODE>(A, beta, R, own);
        if (last_lane) {
            node_load<T, MODE>(A, pold, ex + 1, ey, kk, has_r, R);
            node_value<T, MODE>(A, beta, R, rgt);
        }
        if (last_warp) {
            node_load<T, MODE>(A, pold, ex, ey + 1, kk, has_t, R);
            node_value<T, MODE>(A, beta, R, top);
            if (last_lane) {
                node_load<T, MODE>(A, pold, ex + 1, ey + 1, kk, has_c, R);
                node_value<T, MODE>(A, beta, R, cor);
            }
        }
    };
    // corners (bx + 2 by) of a plane: own and right by shuffle now, the row above
    // from shared memory after the next barrier (collect)
    auto publish = [&](int par, const T (&own)[3], const T (&rgt)[3], const T (&top)[3], const T (&cor)[3],
                       T (&V)[3][4]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T t = __shfl_down_sync(0xffffffffu, own[c], 1);
            const T right = last_lane ? rgt[c] : t;
            S.in[par][w][lane][0][c] = own[c];
            S.in[par][w][lane][1][c] = right;
            V[c][0] = own[c];
            V[c][1] = right;
            const T t2 = __shfl_down_sync(0xffffffffu, top[c], 1);
            V[c][2] = top[c];
            V[c][3] = last_lane ? cor[c] : t2;
        }
    };
    auto collect = [&](int par, T (&V)[3][4]) {
        if (!last_warp) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                V[c][2] = S.in[par][w + 1][lane][0][c];
                V[c][3] = S.in[par][w + 1][lane][1][c];
            }
        }
    };

    // PCG mode: raw inputs of plane kk copied asynchronously into ring stage kk % MV3_STAGES;
    // every thread reads back only its own copies (no barrier needed)
    auto copy_node = [&](int i, int j, int kk, T* dst) {
        const long long n = i + (long long)A.nn[0] * (j + (long long)A.nn[1] * kk);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (sizeof(T) == 4) {
                cp_async4(dst + c, A.r + 3 * n + c);
                cp_async4(dst + 3 + c, pold + 3 * n + c);
            } else {
                cp_async8(dst + c, A.r + 3 * n + c);
                cp_async8(dst + 3 + c, pold + 3 * n + c);
            }
        }
        if (sizeof(T) == 4)
            cp_async4(dst + 6, A.dinv + n);
        else
            cp_async8(dst + 6, A.dinv + n);
    };
    auto issue = [&](int kk) {
        if (kk <= kz1) {
            const int st = kk % MV3_STAGES;
            if (own_xy) copy_node(ex, ey, kk, S.ring.own[st][w][lane]);
            if (has_r) copy_node(ex + 1, ey, kk, S.ring.rgt[st][w]);
            if (has_t) copy_node(ex, ey + 1, kk, S.ring.top[st][lane]);
            if (has_c) copy_node(ex + 1, ey + 1, kk, S.ring.cor[st]);
        }
        cp_async_commit();
    };
    auto raw_value = [&](const T* raw, bool ok, T (&v)[3]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = ok ? fma(beta, raw[3 + c], raw[6] * A.M.kdinv[c] * raw[c]) : T(0);
    };

    T L[3][4], U[3][4];
    {
        T o[3], r_[3] = {T(0), T(0), T(0)}, t[3] = {T(0), T(0), T(0)}, co[3] = {T(0), T(0), T(0)};
        plane_inputs(kz0, o, r_, t, co);
        publish(0, o, r_, t, co, L);
        plane_inputs(kz0 + 1, o, r_, t, co);
        publish(1, o, r_, t, co, U);
        __syncthreads();
        collect(0, L);
        collect(1, U);
        __syncthreads();
    }
    if (MODE == MV_PCG) issue(kz0 + 2);
    T cO[3] = {T(0), T(0), T(0)}, cR[3] = {T(0), T(0), T(0)}, cT[3] = {T(0), T(0), T(0)}, cC[3] = {T(0), T(0), T(0)};
    T dot = T(0);
    for (int k = kz0; k < kz1; ++k) {
        const int par = (k - kz0) & 1;
        // inputs of plane k + 2 (loads issued before the element math)
        T o2[3] = {T(0), T(0), T(0)}, r2[3] = {T(0), T(0), T(0)}, t2[3] = {T(0), T(0), T(0)},
          c2[3] = {T(0), T(0), T(0)};
        const bool more = k + 2 <= kz1;
        if (MODE == MV_PCG)
            issue(k + 3);
        else if (more)
            plane_inputs(k + 2, o2, r2, t2, c2);
        // element (ex, ey, k)
        T y[3][8];
        if (elxy) {
            const T rho = A.escale[ex + (long long)nelx * (ey + (long long)nely * k)];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    y[c][j] = L[c][j];
                    y[c][4 + j] = U[c][j];
                }
            element_apply<T, 3>(A.M, rho, y);
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int j = 0; j < 8; ++j) y[c][j] = T(0);
        }
        // x: right-corner contributions move one lane up
        T col[3][2][2];
#pragma unroll
        for (int by = 0; by < 2; ++by)
#pragma unroll
            for (int bz = 0; bz < 2; ++bz)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T t = __shfl_up_sync(0xffffffffu, y[c][1 + 2 * by + 4 * bz], 1);
                    col[c][by][bz] = y[c][2 * by + 4 * bz] + (lane > 0 ? t : T(0));
                }
        // y: row ey+1 contributions move one warp up; plane k+2 inputs go to the warp below
#pragma unroll
        for (int bz = 0; bz < 2; ++bz)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                S.row[par][w][lane][bz][c] = col[c][1][bz];
                if (last_lane) S.rrow[par][w][bz][c] = y[c][3 + 4 * bz];
            }
        if (MODE == MV_PCG && more) {
            cp_async_wait<1>();   // plane k+2 landed (k+3 may still be in flight)
            const int st = (k + 2) % MV3_STAGES;
            raw_value(S.ring.own[st][w][lane], own_xy, o2);
            if (last_lane) raw_value(S.ring.rgt[st][w], has_r, r2);
            if (last_warp) raw_value(S.ring.top[st][lane], has_t, t2);
            if (last_lane && last_warp) raw_value(S.ring.cor[st], has_c, c2);
        }
        T V2[3][4];
        publish(par, o2, r2, t2, c2, V2);
        __syncthreads();
        collect(par, V2);
        T rowO[2][3], rowR[2][3], rowT[2][3], rowC[2][3];
#pragma unroll
        for (int bz = 0; bz < 2; ++bz)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                rowO[bz][c] = col[c][0][bz] + (w > 0 ? S.row[par][w - 1][lane][bz][c] : T(0));
                rowR[bz][c] = y[c][1 + 4 * bz] + (w > 0 ? S.rrow[par][w - 1][bz][c] : T(0));
                rowT[bz][c] = col[c][1][bz];
                rowC[bz][c] = y[c][3 + 4 * bz];
            }
        // plane k is complete for this tile
        {
            T v[3], pv[3];
            if (own_xy) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c] = cO[c] + rowO[0][c];
                    pv[c] = L[c][0];
                }
                mv3_emit<T, MODE>(A, pnew, 0, ex, ey, k, v, pv, dot);
            }
            if (has_r) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c] = cR[c] + rowR[0][c];
                    pv[c] = L[c][1];
                }
                mv3_emit<T, MODE>(A, pnew, clsx, ex + 1, ey, k, v, pv, dot);
            }
            if (has_t) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c] = cT[c] + rowT[0][c];
                    pv[c] = L[c][2];
                }
                mv3_emit<T, MODE>(A, pnew, clsy, ex, ey + 1, k, v, pv, dot);
            }
            if (has_c) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c] = cC[c] + rowC[0][c];
                    pv[c] = L[c][3];
                }
                mv3_emit<T, MODE>(A, pnew, clsx | clsy, ex + 1, ey + 1, k, v, pv, dot);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cO[c] = rowO[1][c];
            cR[c] = rowR[1][c];
            cT[c] = rowT[1][c];
            cC[c] = rowC[1][c];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                L[c][j] = U[c][j];
                U[c][j] = V2[c][j];
            }
        }
    }
    // top plane of the chunk
    {
        const int clsz = kz1 < nelz ? 4 : 0;
        T pv[3];
        if (own_xy) {
#pragma unroll
            for (int c = 0; c < 3; ++c) pv[c] = L[c][0];
            mv3_emit<T, MODE>(A, pnew, clsz, ex, ey, kz1, cO, pv, dot);
        }
        if (has_r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) pv[c] = L[c][1];
            mv3_emit<T, MODE>(A, pnew, clsx | clsz, ex + 1, ey, kz1, cR, pv, dot);
        }
        if (has_t) {
#pragma unroll
            for (int c = 0; c < 3; ++c) pv[c] = L[c][2];
            mv3_emit<T, MODE>(A, pnew, clsy | clsz, ex, ey + 1, kz1, cT, pv, dot);
        }
        if (has_c) {
#pragma unroll
            for (int c = 0; c < 3; ++c) pv[c] = L[c][3];
            mv3_emit<T, MODE>(A, pnew, clsx | clsy | clsz, ex + 1, ey + 1, kz1, cC, pv, dot);
        }
    }
    if (MODE != MV_PCG) return;
    double v[1] = {(double)dot}, tot[1];
    if (grid_reduce_last<1>(v, A.partials, &A.st->cnt[0], tot)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            A.st->pq = tot[0];
            if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
                A.st->status = 4;
                A.st->done = 1;
            } else {
                A.st->alpha = A.st->rz / tot[0];
            }
        }
    }
}

// PLAIN / RESID epilogue: y = q_final (fixed rows: meandiag x) or r = f - q_final.
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_mv3_finalize(const Mv3Args<T> A, const T* __restrict__ xin,
                                                      T* __restrict__ y, const double* __restrict__ f, T meandiag) {
    double acc = 0.0;
    const long long nnodes = (long long)A.nn[0] * A.nn[1] * A.nn[2];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % A.nn[0]);
        const long long t = n / A.nn[0];
        const int j = (int)(t % A.nn[1]);
        const int k = (int)(t / A.nn[1]);
        T v[3];
        gather_q(A, n, i, j, k, v);
        const unsigned m = A.fixmask[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (MODE == MV_PLAIN) {
                y[3 * n + c] = ((m >> c) & 1u) ? meandiag * xin[3 * n + c] : v[c];
            } else {
                const T rv = ((m >> c) & 1u) ? T(0) : (T)(f[3 * n + c] - (double)v[c]);
                y[3 * n + c] = rv;
                acc += (double)rv * (double)rv;
            }
        }
    }
    if (MODE != MV_RESID) return;
    double v[1] = {acc}, tot[1];
    if (grid_reduce_last<1>(v, A.partials, &A.st->cnt[0], tot))
        if (threadIdx.x == 0) A.st->rr = tot[0];
}

// PCG update for the 3D operator: fixed rows q = meandiag p (= 0), then
// x += alpha p, r -= alpha q, r.z and r.r partials.  q already holds K p: the
// side partials of the tile-boundary nodes were added by k_side_gather3.  The FP32
// dof arrays are streamed as float4 (4 dofs per thread and step), G groups per thread
// and round with every load of the round issued before its first store.
template <typename T, int G = 2>
__global__ void __launch_bounds__(256) k_pcg_update3(const Mv3Args<T> A, T* __restrict__ x, T* __restrict__ r,
                                                     T meandiag, const LoopCond cond) {
    PcgState* st = A.st;
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) loop_cond_set(cond, false);
        return;
    }
    const int it = st->it;
    const T* __restrict__ p = (it & 1) ? A.P1 : A.P0;
    const T* __restrict__ q = A.q;
    const T alpha = (T)st->alpha;
    const unsigned nnodes = (unsigned)A.nn[0] * A.nn[1] * A.nn[2];
    const unsigned ndofs = 3u * nnodes;
    T arz = T(0), arr = T(0);
    if (sizeof(T) == 4) {
        const unsigned nv = ndofs / 4;   // float4 groups; the tail (< 4 dofs) below
        const float4* __restrict__ q4 = reinterpret_cast<const float4*>(q);
        const float4* __restrict__ p4 = reinterpret_cast<const float4*>(p);
        float4* __restrict__ x4 = reinterpret_cast<float4*>(x);
        float4* __restrict__ r4 = reinterpret_cast<float4*>(r);
        const unsigned stride = gridDim.x * blockDim.x;
        auto group = [&](unsigned g, const float4& qv, const float4& pv, const float4& xv, const float4& rv,
                         unsigned m0, unsigned m1, float d0, float d1, unsigned c0) {
            const float qa[4] = {qv.x, qv.y, qv.z, qv.w};
            const float pa[4] = {pv.x, pv.y, pv.z, pv.w};
            const float xa[4] = {xv.x, xv.y, xv.z, xv.w}, ra[4] = {rv.x, rv.y, rv.z, rv.w};
            float xo[4], ro[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const unsigned c = c0 + t;              // 0..5: node n0 (c < 3) or n0 + 1
                const bool second = c >= 3u;
                const unsigned cc = second ? c - 3u : c;
                const unsigned m = second ? m1 : m0;
                const float d = second ? d1 : d0;
                const float kd = (float)A.M.kdinv[cc];
                const float qq = ((m >> cc) & 1u) ? (float)meandiag * pa[t] : qa[t];
                xo[t] = fmaf((float)alpha, pa[t], xa[t]);
                const float rn = fmaf(-(float)alpha, qq, ra[t]);
                ro[t] = rn;
                arz = fmaf(rn, d * kd * rn, arz);
                arr = fmaf(rn, rn, arr);
            }
            x4[g] = make_float4(xo[0], xo[1], xo[2], xo[3]);
            r4[g] = make_float4(ro[0], ro[1], ro[2], ro[3]);
        };
        auto node_of = [&](unsigned g, unsigned& n0, unsigned& nb, unsigned& c0) {
            const unsigned f0 = 4u * g;
            n0 = f0 / 3u;
            c0 = f0 - 3u * n0;
            nb = n0 + 1 < nnodes ? n0 + 1 : n0;
        };
        unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
        for (; g + (G - 1) * stride < nv; g += G * stride) {   // G groups per round, all loads first
            float4 qv[G], pv[G], xv[G], rv[G];
            unsigned n0[G], n1[G], c0[G], m0[G], m1[G];
            float d0[G], d1[G];
#pragma unroll
            for (int k = 0; k < G; ++k) {
                const unsigned gk = g + k * stride;
                node_of(gk, n0[k], n1[k], c0[k]);
                qv[k] = q4[gk];
                pv[k] = p4[gk];
                xv[k] = x4[gk];
                rv[k] = r4[gk];
            }
#pragma unroll
            for (int k = 0; k < G; ++k) {
                m0[k] = A.fixmask[n0[k]];
                m1[k] = A.fixmask[n1[k]];
                d0[k] = (float)A.dinv[n0[k]];
                d1[k] = (float)A.dinv[n1[k]];
            }
#pragma unroll
            for (int k = 0; k < G; ++k) group(g + k * stride, qv[k], pv[k], xv[k], rv[k], m0[k], m1[k], d0[k], d1[k], c0[k]);
        }
        for (; g < nv; g += stride) {
            unsigned na, nab, ca;
            node_of(g, na, nab, ca);
            group(g, q4[g], p4[g], x4[g], r4[g], A.fixmask[na], A.fixmask[nab], (float)A.dinv[na],
                  (float)A.dinv[nab], ca);
        }
        // tail dofs
        for (unsigned f = 4u * nv + blockIdx.x * blockDim.x + threadIdx.x; f < ndofs; f += gridDim.x * blockDim.x) {
            const unsigned n = f / 3u, c = f - 3u * n;
            const unsigned m = A.fixmask[n];
            const T qq = ((m >> c) & 1u) ? meandiag * p[f] : q[f];
            x[f] = fma(alpha, p[f], x[f]);
            const T rn = fma(-alpha, qq, r[f]);
            r[f] = rn;
            arz = fma(rn, A.dinv[n] * A.M.kdinv[c] * rn, arz);
            arr = fma(rn, rn, arr);
        }
    } else {
        for (unsigned f = blockIdx.x * blockDim.x + threadIdx.x; f < ndofs; f += gridDim.x * blockDim.x) {
            const unsigned n = f / 3u, c = f - 3u * n;
            const unsigned m = A.fixmask[n];
            const T qq = ((m >> c) & 1u) ? meandiag * p[f] : q[f];
            x[f] = fma(alpha, p[f], x[f]);
            const T rn = fma(-alpha, qq, r[f]);
            r[f] = rn;
            arz = fma(rn, A.dinv[n] * A.M.kdinv[c] * rn, arz);
            arr = fma(rn, rn, arr);
        }
    }
    double v[2] = {(double)arz, (double)arr}, tot[2];
    if (grid_reduce_last<2>(v, A.partials, &st->cnt[1], tot)) {
        if (threadIdx.x == 0) {
            const double rzo = st->rz;
            st->rz_old = rzo;
            st->rz = tot[0];
            st->beta = rzo != 0.0 ? tot[0] / rzo : 0.0;
            st->rr = tot[1];
            st->it = it + 1;
            if (!isfinite(tot[1])) {
                st->status = 4;
                st->done = 1;
            } else if (tot[1] <= st->tol2) {
                st->status = 0;
                st->done = 1;
            } else if (it + 1 >= st->maxit) {
                st->status = 3;
                st->done = 1;
            } else if (tot[1] < st->ru_delta2 * st->rr_max) {
                st->status = 6;
                st->done = 1;
            }
            st->rr_max = fmax(st->rr_max, tot[1]);
            loop_cond_set(cond, !st->done);
        }
    }
}

// Adds the side partials into q at the tile-boundary nodes (x = 32 m, y = 8 m or
// z = LZ m planes), so that q holds K p before the update streams it.  One
// thread per boundary node; the three plane families are enumerated without
// duplicates (a node on several families is visited once, by its lowest family).
template <typename T>
__global__ void __launch_bounds__(256) k_side_gather3(const Mv3Args<T> A) {
    if (A.st->done) return;
    const int nnx = A.nn[0], nny = A.nn[1], nnz = A.nn[2];
    const long long tx = A.nt[0] - 1, ty = A.nt[1] - 1, tz = A.nt[2] - 1;
    const long long cx = tx * nny * nnz;   // family X: i = 32 mx, all j, k
    const long long cy = ty * nnx * nnz;   // family Y: j = 8 my, i not on an X plane
    const long long cz = tz * nnx * nny;   // family Z: k = LZ mz, i, j not on X / Y planes
    const unsigned tot = (unsigned)(cx + cy + cz);
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
        int i, j, k;
        if (t < (unsigned)cx) {
            const unsigned a = fdiv(t, A.div_nny), b = fdiv(a, A.div_nnz);
            j = (int)(t - a * (unsigned)nny);
            k = (int)(a - b * (unsigned)nnz);
            i = 32 * (int)(b + 1);
        } else if (t < (unsigned)(cx + cy)) {
            const unsigned u = t - (unsigned)cx;
            const unsigned a = fdiv(u, A.div_nnx), b = fdiv(a, A.div_nnz);
            i = (int)(u - a * (unsigned)nnx);
            k = (int)(a - b * (unsigned)nnz);
            j = MV3_BY * (int)(b + 1);
            if ((i & 31) == 0 && i > 0 && i < A.nel[0]) continue;
        } else {
            const unsigned u = t - (unsigned)(cx + cy);
            const unsigned a = fdiv(u, A.div_nnx), b = fdiv(a, A.div_nny);
            i = (int)(u - a * (unsigned)nnx);
            j = (int)(a - b * (unsigned)nny);
            k = A.LZ * (int)(b + 1);
            if ((i & 31) == 0 && i > 0 && i < A.nel[0]) continue;
            if ((j % MV3_BY) == 0 && j > 0 && j < A.nel[1]) continue;
        }
        const bool fx = (i & 31) == 0 && i > 0 && i < A.nel[0];
        const bool fy = (j % MV3_BY) == 0 && j > 0 && j < A.nel[1];
        const bool fz = (k % A.LZ) == 0 && k > 0 && k < A.nel[2];
        const long long n = i + (long long)nnx * (j + (long long)nny * k);
        T v[3] = {T(0), T(0), T(0)};
#pragma unroll 1
        for (int cls = 1; cls < 8; ++cls) {
            const bool on = ((cls & 1) ? fx : true) && ((cls & 2) ? fy : true) && ((cls & 4) ? fz : true);
            if (on) {
                const long long s = side_index(A, cls, i, j, k);
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] += A.side[cls][3 * s + c];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) A.q[3 * n + c] += v[c];
    }
}

}  // namespace tog
