// FP32 PCG operator of 3D structured hex8 grids as a warp march (no shared
// memory, no barriers, no tile-boundary side buffers).
//
// A warp owns one node row y of a strip of 32 node columns (x = 30 cx - 1 + lane;
// lanes 1..30 own their column, lanes 0 and 31 are halo) and marches in z over a
// contiguous range of planes.  For every element plane it applies, in modal form,
// the two elements adjacent to its row (element rows y - 1 and y), keeps only the
// corner forces that land on row y, moves the right-corner forces one lane up by
// shuffle and carries the upper-plane forces to the next step in registers.  The
// element work is doubled (each element is applied by the warps of both of its
// node rows), which buys a kernel with no communication between warps; the
// Hadamard transforms are shared to keep that cost down: the x stage of every
// node row and plane is computed once and carried to the next plane, each element
// adds only its y and z stages, and the inverse transform is taken only to the
// half that lands on row y, the two elements summed before one x stage.  The raw
// inputs of the next planes (r, p_old, D^-1 of rows y - 1, y, y + 1) are loaded
// into a register ring ahead of their use.
//
// Work: items are (column, z band) pairs, band index fastest, handed to the warps
// in strided rounds, so that in every round the warps of adjacent node rows (which
// read each other's rows) and of all bands of a column march in lockstep and the
// shared rows come from L2.  A band's end planes are loaded or applied twice.
//   p = D^-1 r + beta p_old (written for the owned nodes), q = K(rho) p (complete,
//   written for the owned nodes), p.q -> alpha (deterministic grid reduction).
// Fixed dofs need no masking here: r and therefore p are zero there, and the PCG
// update replaces q at fixed dofs by meandiag p.
#pragma once
#include <cuda_runtime.h>

#include "tog_device.cuh"
#include "tog_internal.h"
#include "tog_mv3.cuh"
#include "tog_reduce.cuh"

namespace tog {

constexpr int kM3Warps = 4;   // warps per block
#ifndef TOG_M3_DEPTH
#define TOG_M3_DEPTH 1
#endif
constexpr int kM3Depth = TOG_M3_DEPTH;   // planes loaded ahead

struct M3Row {   // raw operator inputs of one node
    float r[3], po[3], d;
};
struct M3Plane {   // ... of rows y - 1, y, y + 1 of plane j, and the densities of the two
    M3Row row[3];  // elements (rows y - 1 and y) of element plane j - 1
    float rho[2];
};

__global__ void __launch_bounds__(32 * kM3Warps) k_march3(const Mv3Args<float> A, int nstrip, int nband, int lzb) {
    PcgState* st = A.st;
    if (st->done) return;
    constexpr int D = kM3Depth;
    const int it = st->it;
    float* __restrict__ pnew = (it & 1) ? A.P1 : A.P0;
    const float* __restrict__ pold = (it & 1) ? A.P0 : A.P1;
    const float beta = (float)st->beta;
    const int lane = threadIdx.x & 31;
    // 32-bit index arithmetic: the handle keeps 3 x nodes below 2^31
    const int GW = gridDim.x * kM3Warps;
    const int gw = blockIdx.x * kM3Warps + (threadIdx.x >> 5);
    const int nnx = A.nn[0], nny = A.nn[1], nnz = A.nn[2], nelx = A.nel[0], nely = A.nel[1], nelz = A.nel[2];
    const unsigned plane = (unsigned)nnx * (unsigned)nny;
    const int items = nstrip * nny * nband;   // (column, z band), band fastest
    float dot = 0.f;
    for (int t = gw; t < items; t += GW) {
        const int col = t / nband;
        const int band = (int)(t - col * nband);
        const int za = band * lzb;
        const int zb = za + lzb < nnz ? za + lzb : nnz;
        if (za >= zb) continue;
        const int y = (int)(col % nny), cx = (int)(col / nny);
        const int x = 30 * cx - 1 + lane;
        const bool colok = x >= 0 && x < nnx;
        const bool elx = x >= 0 && x < nelx && lane < 31;
        const bool own = colok && lane >= 1 && lane <= 30;
        const bool e0ok = y >= 1 && y - 1 < nely, e1ok = y < nely;
        bool rok[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) rok[r] = colok && y - 1 + r >= 0 && y - 1 + r < nny;
        const unsigned xu = (unsigned)x;   // used only where the node exists (x >= 0)
        auto load = [&](int j, M3Plane& R) {
            const bool pok = j >= 0 && j < nnz;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const bool ok = rok[r] && pok;
                const unsigned n = ok ? xu + (unsigned)nnx * (unsigned)(y - 1 + r) + plane * (unsigned)j : 0u;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    R.row[r].r[c] = ok ? A.r[3 * n + c] : 0.f;
                    R.row[r].po[c] = ok ? pold[3 * n + c] : 0.f;
                }
                R.row[r].d = ok ? A.dinv[n] : 0.f;
            }
            const int ez = j - 1;
            const bool zok = elx && ez >= 0 && ez < nelz;
            const unsigned e1 = xu + (unsigned)nelx * ((unsigned)y + (unsigned)nely * (unsigned)ez);
            R.rho[0] = (zok && e0ok) ? A.escale[e1 - (unsigned)nelx] : 0.f;
            R.rho[1] = (zok && e1ok) ? A.escale[e1] : 0.f;
        };
        const int j0 = za - 1, j1 = zb;   // planes walked (inclusive)
        M3Plane buf[D];
#pragma unroll
        for (int q = 0; q < D; ++q)
            if (j0 + q <= j1) load(j0 + q, buf[q]);
        // Carried state: x stage of the lower plane's Hadamard transform for rows
        // y - 1, y, y + 1 (XL[row][mx][c] = own + right, right - own), its p on row y,
        // and the forces on row y of the current plane from the element plane below.
        float XL[3][2][3], pl1[3] = {0.f, 0.f, 0.f}, cO[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) XL[r][0][c] = XL[r][1][c] = 0.f;
        for (int jb = j0; jb <= j1; jb += D) {
#pragma unroll
            for (int q = 0; q < D; ++q) {
                const int j = jb + q;
                if (j > j1) break;
                float XU[3][2][3], p1[3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float pv =
                            fmaf(beta, buf[q].row[r].po[c], buf[q].row[r].d * A.M.kdinv[c] * buf[q].row[r].r[c]);
                        const float pr = __shfl_down_sync(0xffffffffu, pv, 1);
                        XU[r][0][c] = pv + pr;
                        XU[r][1][c] = pr - pv;
                        if (r == 1) p1[c] = pv;
                    }
                const float rho2[2] = {buf[q].rho[0], buf[q].rho[1]};
                if (j + D <= j1) load(j + D, buf[q]);
                if (j >= za) {   // element plane j - 1: forces on row y of planes j - 1 and j
                    const int ez = j - 1;
                    const bool ezok = ez >= 0 && ez < nelz;
                    float S[4][3];   // inverse transform of both elements up to the x stage (bits x, z)
#pragma unroll
                    for (int i = 0; i < 4; ++i) S[i][0] = S[i][1] = S[i][2] = 0.f;
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        if (!((e == 0 ? e0ok : e1ok) && ezok)) continue;   // warp-uniform
                        const float rho = rho2[e];
                        // forward y and z stages (mode m = mx + 2 my + 4 mz)
                        float u[3][8], bm[3][8];
#pragma unroll
                        for (int mx = 0; mx < 2; ++mx)
#pragma unroll
                            for (int c = 0; c < 3; ++c) {
                                const float lo0 = XL[e][mx][c] + XL[e + 1][mx][c];
                                const float lo1 = XL[e + 1][mx][c] - XL[e][mx][c];
                                const float up0 = XU[e][mx][c] + XU[e + 1][mx][c];
                                const float up1 = XU[e + 1][mx][c] - XU[e][mx][c];
                                u[c][mx] = lo0 + up0;
                                u[c][mx + 4] = up0 - lo0;
                                u[c][mx + 2] = lo1 + up1;
                                u[c][mx + 6] = up1 - lo1;
                            }
                        modal_mul<float, 3>(A.M, rho, u, bm);
                        // inverse z stage, then the half of the y stage on row y
                        // (by = 1 for element row y - 1, by = 0 for element row y)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            float w[8];
#pragma unroll
                            for (int m = 0; m < 4; ++m) {
                                w[m] = bm[c][m] - bm[c][m + 4];
                                w[m + 4] = bm[c][m] + bm[c][m + 4];
                            }
                            const int idx[4] = {0, 1, 4, 5};
#pragma unroll
                            for (int t = 0; t < 4; ++t) {
                                const int i = idx[t];
                                S[t][c] += (e == 0) ? w[i] + w[i + 2] : w[i] - w[i + 2];
                            }
                        }
                    }
                    float qlo[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        // inverse x stage: own / right corner on the lower and upper plane
                        const float oL = S[0][c] - S[1][c], rL = S[0][c] + S[1][c];
                        const float oU = S[2][c] - S[3][c], rU = S[2][c] + S[3][c];
                        const float tL = __shfl_up_sync(0xffffffffu, rL, 1);
                        const float tU = __shfl_up_sync(0xffffffffu, rU, 1);
                        qlo[c] = cO[c] + oL + (lane > 0 ? tL : 0.f);
                        cO[c] = oU + (lane > 0 ? tU : 0.f);
                    }
                    if (j > za && own) {   // node (x, y, j - 1) is complete
                        const unsigned n = xu + (unsigned)nnx * (unsigned)y + plane * (unsigned)(j - 1);
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            pnew[3 * n + c] = pl1[c];
                            A.q[3 * n + c] = qlo[c];
                            dot = fmaf(pl1[c], qlo[c], dot);
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        XL[r][0][c] = XU[r][0][c];
                        XL[r][1][c] = XU[r][1][c];
                    }
#pragma unroll
                for (int c = 0; c < 3; ++c) pl1[c] = p1[c];
            }
        }
    }
    double v[1] = {(double)dot}, tot[1];
    if (grid_reduce_last<1>(v, A.partials, &st->cnt[0], tot)) {
        if (threadIdx.x == 0) {
            st->pq = tot[0];
            if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
                st->status = 4;
                st->done = 1;
            } else {
                st->alpha = st->rz / tot[0];
            }
        }
    }
}

}  // namespace tog
