// FP32 3D hex8 operator with packed f32x2 arithmetic (sm_103a).
//
// Same tiling, node ownership and side-buffer classes as k_mv3 (32 x 8 element
// tiles, LZ-layer z chunks, see tog_mv3.cuh), so the same consumers
// (k_pcg_update3, k_mv3_finalize) read its output.  The work split differs:
// each thread owns an x-pair of elements, A = (ex0, ey) and B = (ex0+1, ey),
// and a warp covers 16 pairs x 2 rows.  The pair's middle node column stays in
// registers, neighbour exchanges halve, and the Hadamard stages of both
// elements run as one packed f32x2 instruction stream (.x = A, .y = B).
#pragma once
#include "tog_mv3.cuh"

namespace tog {

constexpr int MX_WARPS = 4;   // 4 warps x 2 rows = 8 element rows per tile (= MV3_BY)
static_assert(2 * MX_WARPS == MV3_BY, "tile height must match the side-buffer layout");

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

struct Mx2Smem {
    float2 own[2][9][16][3];            // plane inputs by row slot (8 = halo row): own pair
    float rgt[2][9][16][3];             //   ... and the right neighbour value
    float2 row[2][MX_WARPS][16][2][3];  // output row ey+1 of the hy = 1 lanes, for the next warp
    float rrow[2][MX_WARPS][2][3];      // the same for the right halo column (hx = 15)
};

struct PlaneV {
    float2 own[3];   // nodes (ex0, ey), (ex0+1, ey)
    float rgt[3];    // node (ex0+2, ey)
    float2 town[3];  // nodes (ex0, ey+1), (ex0+1, ey+1)
    float trgt[3];   // node (ex0+2, ey+1)
};

template <int MODE>
__device__ __forceinline__ float x2_node(const Mv3Args<float>& A, const float* __restrict__ pold, float beta,
                                         unsigned n, bool ok, int c) {
    if (!ok) return 0.f;
    if (MODE == MV_PCG) return fmaf(beta, pold[3u * n + c], A.dinv[n] * A.M.kdinv[c] * A.r[3u * n + c]);
    return ((A.fixmask[n] >> c) & 1u) ? 0.f : A.x[3u * n + c];
}

template <int MODE>
__device__ __forceinline__ void x2_emit(const Mv3Args<float>& A, float* __restrict__ pnew, int cls, int i, int j,
                                        int k, float v, float pv, int c, float& dot) {
    if (cls == 0) {
        const unsigned n = (unsigned)i + (unsigned)A.nn[0] * ((unsigned)j + (unsigned)A.nn[1] * (unsigned)k);
        A.q[3u * n + c] = v;
        if (MODE == MV_PCG) pnew[3u * n + c] = pv;
    } else {
        const long long s = side_index(A, cls, i, j, k);
        A.side[cls][3 * s + c] = v;
    }
    if (MODE == MV_PCG) dot = fmaf(pv, v, dot);
}

template <int MODE>
__global__ void __launch_bounds__(32 * MX_WARPS, 3) k_mv3x2(const Mv3Args<float> A) {
    __shared__ __align__(16) Mx2Smem S;
    const int lane = threadIdx.x, w = threadIdx.y;
    const int hx = lane & 15, hy = lane >> 4;
    float beta = 0.f;
    const float* __restrict__ pold = nullptr;
    float* __restrict__ pnew = nullptr;
    if (MODE == MV_PCG) {
        if (A.st->done) return;
        const int it = A.st->it;
        pnew = (it & 1) ? A.P1 : A.P0;
        pold = (it & 1) ? A.P0 : A.P1;
        beta = (float)A.st->beta;
    }
    const int nelx = A.nel[0], nely = A.nel[1], nelz = A.nel[2];
    const unsigned nnx = A.nn[0], plane = (unsigned)A.nn[0] * A.nn[1];
    const int ex0 = 32 * (int)blockIdx.x + 2 * hx;
    const int ey = MV3_BY * (int)blockIdx.y + 2 * w + hy;
    const int slot = 2 * w + hy;
    const int kz0 = A.LZ * (int)blockIdx.z;
    const int kz1 = min(kz0 + A.LZ, nelz);
    const bool eA = ex0 < nelx && ey < nely, eB = ex0 + 1 < nelx && ey < nely;
    const bool ok0 = ex0 <= nelx && ey <= nely, ok1 = ex0 + 1 <= nelx && ey <= nely;
    const bool rx = hx == 15, tp = (w == MX_WARPS - 1) && hy == 1;
    const bool okr = rx && ex0 + 2 <= nelx && ey <= nely;
    const bool okt0 = tp && ey + 1 <= nely && ex0 <= nelx, okt1 = tp && ey + 1 <= nely && ex0 + 1 <= nelx;
    const bool okc = tp && rx && ey + 1 <= nely && ex0 + 2 <= nelx;
    const int clsx = (32 * ((int)blockIdx.x + 1) < nelx) ? 1 : 0;
    const int clsy = (MV3_BY * ((int)blockIdx.y + 1) < nely) ? 2 : 0;
    const unsigned nrow = (unsigned)ex0 + nnx * (unsigned)ey;   // node (ex0, ey) of plane 0

    // operator input at this thread's nodes of plane kk, published for the row below
    auto inputs = [&](int kk, int par, PlaneV& V) {
        const unsigned n = nrow + plane * (unsigned)kk;
        float2 tw[3];
        float tr[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            V.own[c] = make_float2(x2_node<MODE>(A, pold, beta, n, ok0, c), x2_node<MODE>(A, pold, beta, n + 1, ok1, c));
            V.rgt[c] = x2_node<MODE>(A, pold, beta, n + 2, okr, c);   // halo duty only (hx = 15)
            tw[c] = make_float2(x2_node<MODE>(A, pold, beta, n + nnx, okt0, c),
                                x2_node<MODE>(A, pold, beta, n + nnx + 1, okt1, c));
            tr[c] = x2_node<MODE>(A, pold, beta, n + nnx + 2, okc, c);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float sr = __shfl_down_sync(0xffffffffu, V.own[c].x, 1);
            const float st = __shfl_down_sync(0xffffffffu, tw[c].x, 1);
            if (!rx) V.rgt[c] = sr;
            if (!rx) tr[c] = st;
            S.own[par][slot][hx][c] = V.own[c];
            S.rgt[par][slot][hx][c] = V.rgt[c];
            if (tp) {
                S.own[par][8][hx][c] = tw[c];
                S.rgt[par][8][hx][c] = tr[c];
            }
        }
    };
    auto collect = [&](int par, PlaneV& V) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            V.town[c] = S.own[par][slot + 1][hx][c];
            V.trgt[c] = S.rgt[par][slot + 1][hx][c];
        }
    };

    PlaneV L, U;
    inputs(kz0, 0, L);
    inputs(kz0 + 1, 1, U);
    __syncthreads();
    collect(0, L);
    collect(1, U);
    __syncthreads();

    float2 cO[3], cT[3];
    float cR[3], cC[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        cO[c] = cT[c] = make_float2(0.f, 0.f);
        cR[c] = cC[c] = 0.f;
    }
    float dot = 0.f;
    for (int k = kz0; k < kz1; ++k) {
        const int par = (k - kz0) & 1;
        PlaneV V2;
        const bool more = k + 2 <= kz1;
        if (more) {
            inputs(k + 2, par, V2);
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                V2.own[c] = V2.town[c] = make_float2(0.f, 0.f);
                V2.rgt[c] = V2.trgt[c] = 0.f;
            }
        }
        // ---- element pair (A, B) at layer k
        float2 rho = make_float2(0.f, 0.f);
        {
            const unsigned e = (unsigned)ex0 + (unsigned)nelx * ((unsigned)ey + (unsigned)nely * (unsigned)k);
            if (eA) rho.x = A.escale[e];
            if (eB) rho.y = A.escale[e + 1];
        }
        float2 y[3][8];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            y[c][0] = L.own[c];
            y[c][1] = make_float2(L.own[c].y, L.rgt[c]);
            y[c][2] = L.town[c];
            y[c][3] = make_float2(L.town[c].y, L.trgt[c]);
            y[c][4] = U.own[c];
            y[c][5] = make_float2(U.own[c].y, U.rgt[c]);
            y[c][6] = U.town[c];
            y[c][7] = make_float2(U.town[c].y, U.trgt[c]);
            // forward Hadamard (packed): stages x, y, z
#pragma unroll
            for (int s = 1; s < 8; s <<= 1)
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (!(i & s)) {
                        const float2 a = y[c][i], b = y[c][i + s];
                        y[c][i] = f2add(a, b);
                        y[c][i + s] = f2sub(b, a);
                    }
            // scale the element pair by (rho_A, rho_B)
#pragma unroll
            for (int m = 1; m < 8; ++m) y[c][m] = __fmul2_rn(y[c][m], rho);
        }
        // modal product (scalar constants from the parameter bank)
        float2 b[3][8];
#pragma unroll
        for (int c = 0; c < 3; ++c) b[c][0] = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 1; m < 8; ++m)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float ax = A.M.D[m][c] * y[c][m].x, ay = A.M.D[m][c] * y[c][m].y;
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (d != c && (((m >> c) & 1) != ((m >> d) & 1))) {
                        const int mm = m ^ (1 << c) ^ (1 << d);
                        ax = fmaf(A.M.O[m][c][d], y[d][mm].x, ax);
                        ay = fmaf(A.M.O[m][c][d], y[d][mm].y, ay);
                    }
                b[c][m] = make_float2(ax, ay);
            }
        // inverse Hadamard (packed)
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int s = 4; s > 0; s >>= 1)
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (!(i & s)) {
                        const float2 a = b[c][i], bb = b[c][i + s];
                        b[c][i] = f2sub(a, bb);
                        b[c][i + s] = f2add(a, bb);
                    }
        // ---- x: pair-internal middle node, left neighbour's right corner by shuffle
        float2 out[2][2][3];   // [by][bz][c]: nodes (ex0, ex0+1)
        float rs[2][2][3];     // right corner of B (node ex0+2), kept for the halo column
#pragma unroll
        for (int by = 0; by < 2; ++by)
#pragma unroll
            for (int bz = 0; bz < 2; ++bz)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float2 Y0 = b[c][2 * by + 4 * bz], Y1 = b[c][1 + 2 * by + 4 * bz];
                    const float rv = __shfl_up_sync(0xffffffffu, Y1.y, 1);
                    out[by][bz][c] = make_float2(Y0.x + (hx > 0 ? rv : 0.f), Y1.x + Y0.y);
                    rs[by][bz][c] = Y1.y;
                }
        // ---- y: hy 0 -> 1 by shuffle, hy 1 -> next warp through shared memory
        float2 up_o[2][3];
        float up_r[2][3];
#pragma unroll
        for (int bz = 0; bz < 2; ++bz)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                up_o[bz][c].x = __shfl_up_sync(0xffffffffu, out[1][bz][c].x, 16);
                up_o[bz][c].y = __shfl_up_sync(0xffffffffu, out[1][bz][c].y, 16);
                up_r[bz][c] = __shfl_up_sync(0xffffffffu, rs[1][bz][c], 16);
                if (hy == 1) {
                    S.row[par][w][hx][bz][c] = out[1][bz][c];
                    if (rx) S.rrow[par][w][bz][c] = rs[1][bz][c];
                }
            }
        __syncthreads();
        if (more) collect(par, V2);
        float2 rowO[2][3];
        float rowR[2][3];
#pragma unroll
        for (int bz = 0; bz < 2; ++bz)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float2 addo = make_float2(0.f, 0.f);
                float addr = 0.f;
                if (hy == 1) {
                    addo = up_o[bz][c];
                    addr = up_r[bz][c];
                } else if (w > 0) {
                    addo = S.row[par][w - 1][hx][bz][c];
                    addr = S.rrow[par][w - 1][bz][c];
                }
                rowO[bz][c] = f2add(out[0][bz][c], addo);
                rowR[bz][c] = rs[0][bz][c] + addr;
            }
        // ---- plane k complete for this tile: emit
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 v = f2add(cO[c], rowO[0][c]);
            if (ok0) x2_emit<MODE>(A, pnew, 0, ex0, ey, k, v.x, L.own[c].x, c, dot);
            if (ok1) x2_emit<MODE>(A, pnew, 0, ex0 + 1, ey, k, v.y, L.own[c].y, c, dot);
            if (okr) x2_emit<MODE>(A, pnew, clsx, ex0 + 2, ey, k, cR[c] + rowR[0][c], L.rgt[c], c, dot);
            if (tp) {
                const float2 vt = f2add(cT[c], out[1][0][c]);
                if (okt0) x2_emit<MODE>(A, pnew, clsy, ex0, ey + 1, k, vt.x, L.town[c].x, c, dot);
                if (okt1) x2_emit<MODE>(A, pnew, clsy, ex0 + 1, ey + 1, k, vt.y, L.town[c].y, c, dot);
                if (okc) x2_emit<MODE>(A, pnew, clsx | clsy, ex0 + 2, ey + 1, k, cC[c] + rs[1][0][c], L.trgt[c], c, dot);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cO[c] = rowO[1][c];
            cR[c] = rowR[1][c];
            cT[c] = out[1][1][c];
            cC[c] = rs[1][1][c];
        }
        L = U;
        U = V2;
    }
    // top plane of the chunk
    {
        const int clsz = kz1 < nelz ? 4 : 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (ok0) x2_emit<MODE>(A, pnew, clsz, ex0, ey, kz1, cO[c].x, L.own[c].x, c, dot);
            if (ok1) x2_emit<MODE>(A, pnew, clsz, ex0 + 1, ey, kz1, cO[c].y, L.own[c].y, c, dot);
            if (okr) x2_emit<MODE>(A, pnew, clsx | clsz, ex0 + 2, ey, kz1, cR[c], L.rgt[c], c, dot);
            if (tp) {
                if (okt0) x2_emit<MODE>(A, pnew, clsy | clsz, ex0, ey + 1, kz1, cT[c].x, L.town[c].x, c, dot);
                if (okt1) x2_emit<MODE>(A, pnew, clsy | clsz, ex0 + 1, ey + 1, kz1, cT[c].y, L.town[c].y, c, dot);
                if (okc) x2_emit<MODE>(A, pnew, clsx | clsy | clsz, ex0 + 2, ey + 1, kz1, cC[c], L.trgt[c], c, dot);
            }
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

}  // namespace tog
