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
// node rows), which buys a kernel with no communication between warps.  The raw
// inputs of the next planes (r, p_old, D^-1 of rows y - 1, y, y + 1) are loaded
// into a register ring ahead of their use.
//
// Work: the (column, plane) steps, ordered column-major in z, are split into one
// contiguous range per warp; a range crosses columns in segments, and only a
// segment's end planes are loaded or applied twice.
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
constexpr int kM3Depth = 2;   // planes loaded ahead

struct M3Row {   // raw operator inputs of one node
    float r[3], po[3], d;
};

__global__ void __launch_bounds__(32 * kM3Warps) k_march3(const Mv3Args<float> A, int nstrip) {
    PcgState* st = A.st;
    if (st->done) return;
    constexpr int D = kM3Depth;
    const int it = st->it;
    float* __restrict__ pnew = (it & 1) ? A.P1 : A.P0;
    const float* __restrict__ pold = (it & 1) ? A.P0 : A.P1;
    const float beta = (float)st->beta;
    const int lane = threadIdx.x & 31;
    const long long GW = (long long)gridDim.x * kM3Warps;
    const long long gw = (long long)blockIdx.x * kM3Warps + (threadIdx.x >> 5);
    const int nnx = A.nn[0], nny = A.nn[1], nnz = A.nn[2], nelx = A.nel[0], nely = A.nel[1], nelz = A.nel[2];
    const long long plane = (long long)nnx * nny;
    const long long total = (long long)nstrip * nny * nnz;   // (column, plane) steps
    long long s = total * gw / GW;
    const long long s1 = total * (gw + 1) / GW;
    float dot = 0.f;
    while (s < s1) {
        const long long col = s / nnz;
        const int za = (int)(s - col * nnz);
        const int zb = (int)((s1 - s) < (long long)(nnz - za) ? za + (s1 - s) : nnz);
        s += zb - za;
        const int y = (int)(col % nny), cx = (int)(col / nny);
        const int x = 30 * cx - 1 + lane;
        const bool colok = x >= 0 && x < nnx;
        const bool elx = x >= 0 && x < nelx && lane < 31;
        const bool own = colok && lane >= 1 && lane <= 30;
        const bool e0ok = y >= 1 && y - 1 < nely, e1ok = y < nely;
        bool rok[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) rok[r] = colok && y - 1 + r >= 0 && y - 1 + r < nny;
        const long long nb = x + (long long)nnx * (y - 1);   // node (x, y - 1, 0)
        auto load = [&](int j, M3Row (&R)[3]) {
            const bool pok = j >= 0 && j < nnz;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const bool ok = rok[r] && pok;
                const long long n = ok ? nb + (long long)nnx * r + plane * j : 0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    R[r].r[c] = ok ? A.r[3 * n + c] : 0.f;
                    R[r].po[c] = ok ? pold[3 * n + c] : 0.f;
                }
                R[r].d = ok ? A.dinv[n] : 0.f;
            }
        };
        const int j0 = za - 1, j1 = zb;   // planes walked (inclusive)
        M3Row buf[D][3];
#pragma unroll
        for (int q = 0; q < D; ++q)
            if (j0 + q <= j1) load(j0 + q, buf[q]);
        float plo[3][3], cO[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int r = 0; r < 3; ++r) plo[r][0] = plo[r][1] = plo[r][2] = 0.f;
        for (int jb = j0; jb <= j1; jb += D) {
#pragma unroll
            for (int q = 0; q < D; ++q) {
                const int j = jb + q;
                if (j > j1) break;
                float pj[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        pj[r][c] = fmaf(beta, buf[q][r].po[c], buf[q][r].d * A.M.kdinv[c] * buf[q][r].r[c]);
                if (j + D <= j1) load(j + D, buf[q]);
                if (j >= za) {   // element plane j - 1: forces on row y of planes j - 1 and j
                    const int ez = j - 1;
                    const bool ezok = ez >= 0 && ez < nelz;
                    float oL[3] = {0.f, 0.f, 0.f}, rL[3] = {0.f, 0.f, 0.f}, oU[3] = {0.f, 0.f, 0.f},
                          rU[3] = {0.f, 0.f, 0.f};
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        if (!((e == 0 ? e0ok : e1ok) && ezok)) continue;   // warp-uniform
                        const int ey = y - 1 + e;
                        const float rho = elx ? A.escale[x + (long long)nelx * (ey + (long long)nely * ez)] : 0.f;
                        float yv[3][8];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            yv[c][0] = plo[e][c];
                            yv[c][1] = __shfl_down_sync(0xffffffffu, plo[e][c], 1);
                            yv[c][2] = plo[e + 1][c];
                            yv[c][3] = __shfl_down_sync(0xffffffffu, plo[e + 1][c], 1);
                            yv[c][4] = pj[e][c];
                            yv[c][5] = __shfl_down_sync(0xffffffffu, pj[e][c], 1);
                            yv[c][6] = pj[e + 1][c];
                            yv[c][7] = __shfl_down_sync(0xffffffffu, pj[e + 1][c], 1);
                        }
                        element_apply<float, 3>(A.M, rho, yv);
                        const int b = (e == 0) ? 2 : 0;   // corners on node row y
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            oL[c] += yv[c][b];
                            rL[c] += yv[c][b + 1];
                            oU[c] += yv[c][b + 4];
                            rU[c] += yv[c][b + 5];
                        }
                    }
                    float qlo[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float tL = __shfl_up_sync(0xffffffffu, rL[c], 1);
                        const float tU = __shfl_up_sync(0xffffffffu, rU[c], 1);
                        qlo[c] = cO[c] + oL[c] + (lane > 0 ? tL : 0.f);
                        cO[c] = oU[c] + (lane > 0 ? tU : 0.f);
                    }
                    if (j > za && own) {   // node (x, y, j - 1) is complete
                        const long long n = nb + nnx + plane * (j - 1);
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            pnew[3 * n + c] = plo[1][c];
                            A.q[3 * n + c] = qlo[c];
                            dot = fmaf(plo[1][c], qlo[c], dot);
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) plo[r][c] = pj[r][c];
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
