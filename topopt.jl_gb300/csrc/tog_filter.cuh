// Node-based density filter J = M2 M1 and its transpose as shared-memory stencils
// (src/CheqFilters/density_filter.jl:25-121 with the neighbour weights of
// CheqFilters.jl:66-118: every node within rmin of a cell centre weighs
// (rmin - d) * valence(node)).
//
// A block owns a tile of kFiltTX x kFiltTY cells and walks a band of its cell
// planes in z (2D: the tile alone).  Forward: each step loads one cell plane of
// the tile and its halo into shared memory, averages it onto one plane of nodes
// (M1: the mean of the cells around a node), keeps the last nz node planes of the
// stencil's z reach in a shared ring, and forms one output cell plane from them
// (M2: y_e = invW_e sum_s w_s valence(n) nodal_n).  Transpose: each step loads one
// plane of invW d, accumulates one node plane of M2' (valence(n) sum_s w_s
// (invW d)_{n - off_s}) from a shared ring of those planes, and forms one output
// cell plane from the two latest node planes (M1': sum over the corners of
// nodal_n / valence(n)).  The nodal intermediate never leaves the SM.  Both kernels
// are bound by the FP64 pipe (GB300 runs FP64 at a small fraction of its FP32 rate),
// so they skip the valence factors, which cancel exactly (below).
#pragma once
#include <cuda_runtime.h>

#include "tog_device.cuh"
#include "tog_internal.h"

namespace tog {

constexpr int kFiltTX = 32, kFiltTY = 8;   // cell tile of a block (one thread per cell column)
constexpr size_t kFiltMaxSmem = 200 * 1024;  // larger stencils run the two-pass kernels

// Range of the stencil's node offsets (from a cell's lower corner node) per axis.
struct FiltBox {
    int lo[3], hi[3];
};

// Shared memory of the forward kernel: stencil, cell ring (2 planes), node ring (nz planes).
inline size_t filt_fwd_smem(const FiltBox& B, int S, int dim) {
    const int nxn = kFiltTX + B.hi[0] - B.lo[0], nyn = kFiltTY + B.hi[1] - B.lo[1];
    const int nzr = dim == 3 ? B.hi[2] - B.lo[2] + 1 : 1;
    return sizeof(double) * ((size_t)2 * (nxn + 1) * (nyn + 1) + (size_t)nzr * nxn * nyn + S) + sizeof(int) * 3 * S;
}
// ... of the transpose: stencil, ring of nz planes of invW d, node ring (2 planes).
inline size_t filt_bwd_smem(const FiltBox& B, int S, int dim) {
    const int nxc = kFiltTX + 1 + B.hi[0] - B.lo[0], nyc = kFiltTY + 1 + B.hi[1] - B.lo[1];
    const int nzr = dim == 3 ? B.hi[2] - B.lo[2] + 1 : 1;
    return sizeof(double) * ((size_t)nzr * nxc * nyc + (size_t)2 * (kFiltTX + 1) * (kFiltTY + 1) + S) +
           sizeof(int) * 3 * S;
}

// The valence of a node of a structured grid (the number of cells around it) is a power
// of two and equals the number of cells its average is taken over, so the reference's
// w_s * valence(n) * (sum / valence(n)) equals w_s * sum bit for bit (scaling by a power
// of two is exact); the transpose's valence(n) * acc / valence(n) likewise equals acc.
// The kernels therefore carry nodal sums, not means, and apply no valence at all.

__device__ __forceinline__ int pmod(int a, int m) {
    const int r = a % m;
    return r < 0 ? r + m : r;
}

// y = J x.  Grid: (x tiles, y tiles, z bands of lz cell planes).  An element whose ball
// holds no node keeps its input (invW = 0), as the reference skips the row.
template <int DIM>
__global__ void __launch_bounds__(kFiltTX * kFiltTY) k_filt_fwd(const double* __restrict__ x, double* __restrict__ y,
                                                               const int* __restrict__ soff,
                                                               const double* __restrict__ sw, int S,
                                                               const double* __restrict__ invW, Dims D, FiltBox B,
                                                               int lz) {
    extern __shared__ double fsm[];
    const int nxn = kFiltTX + B.hi[0] - B.lo[0], nyn = kFiltTY + B.hi[1] - B.lo[1];
    const int nxc = nxn + 1, nyc = nyn + 1;
    const int nzr = DIM == 3 ? B.hi[2] - B.lo[2] + 1 : 1;
    double* cells = fsm;                          // [2][nyc][nxc]
    double* nodal = cells + 2 * nxc * nyc;        // [nzr][nyn][nxn]
    double* w = nodal + nzr * nxn * nyn;          // [S]
    int* off = reinterpret_cast<int*>(w + S);     // [S][3]
    const int tid = threadIdx.x, nth = blockDim.x;
    const int tx = tid % kFiltTX, ty = tid / kFiltTX;
    for (int s = tid; s < S; s += nth) {
        w[s] = sw[s];
        off[3 * s] = soff[3 * s];
        off[3 * s + 1] = soff[3 * s + 1];
        off[3 * s + 2] = soff[3 * s + 2];
    }
    const int ex0 = blockIdx.x * kFiltTX, ey0 = blockIdx.y * kFiltTY;
    const int nx0 = ex0 + B.lo[0], ny0 = ey0 + B.lo[1];   // first node of the tile's node window
    const int cx0 = nx0 - 1, cy0 = ny0 - 1;               // first cell of its cell window
    const int za = DIM == 3 ? blockIdx.z * lz : 0;
    const int zb = DIM == 3 ? min(za + lz, D.nel[2]) : 1;
    const long long cplane = (long long)D.nel[0] * D.nel[1];
    auto load_cells = [&](int cz, double* dst) {
        const bool zok = DIM == 2 || (cz >= 0 && cz < D.nel[2]);
        for (int ay = ty; ay < nyc; ay += kFiltTY)
            for (int ax = tx; ax < nxc; ax += kFiltTX) {
                const int cx = cx0 + ax, cy = cy0 + ay;
                const bool ok = zok && cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1];
                dst[ay * nxc + ax] = ok ? x[cx + (long long)D.nel[0] * cy + cplane * (DIM == 3 ? cz : 0)] : 0.0;
            }
    };
    // node plane iz from cell planes iz - 1 (lo) and iz (hi) of the cell ring
    auto make_nodes = [&](int iz, const double* clo, const double* chi, double* dst) {
        for (int ay = ty; ay < nyn; ay += kFiltTY)
          for (int ax = tx; ax < nxn; ax += kFiltTX) {
            const int ix = nx0 + ax, iy = ny0 + ay;
            double s = 0.0;
#pragma unroll
            for (int bz = 0; bz < (DIM == 3 ? 2 : 1); ++bz) {
                const int cz = iz - 1 + bz;
                if (DIM == 3 && (cz < 0 || cz >= D.nel[2])) continue;
                const double* c = (DIM == 3 && bz == 0) ? clo : chi;
#pragma unroll
                for (int by = 0; by < 2; ++by)
#pragma unroll
                    for (int bx = 0; bx < 2; ++bx) {
                        const int cx = ix - 1 + bx, cy = iy - 1 + by;
                        if (cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1]) s += c[(ay + by) * nxc + (ax + bx)];
                    }
            }
            dst[ay * nxn + ax] = s;
          }
    };
    auto out_plane = [&](int ez) {
        {
            const int ex = ex0 + tx, ey = ey0 + ty;
            if (ex >= D.nel[0] || ey >= D.nel[1]) return;
            const long long e = ex + (long long)D.nel[0] * ey + cplane * ez;
            double acc = 0.0;
            for (int s = 0; s < S; ++s) {
                const int ix = ex + off[3 * s], iy = ey + off[3 * s + 1], iz = ez + off[3 * s + 2];
                if (ix < 0 || ix >= D.nn[0] || iy < 0 || iy >= D.nn[1] ||
                    (DIM == 3 && (iz < 0 || iz >= D.nn[2])))
                    continue;
                const double* np = nodal + (DIM == 3 ? pmod(iz, nzr) : 0) * nxn * nyn;
                acc += w[s] * np[(iy - ny0) * nxn + (ix - nx0)];
            }
            const double iw = invW[e];
            y[e] = iw > 0.0 ? acc * iw : x[e];
        }
    };
    if (DIM == 2) {
        load_cells(0, cells);
        __syncthreads();
        make_nodes(0, cells, cells, nodal);
        __syncthreads();
        out_plane(0);
        return;
    }
    if (za >= zb) return;   // uniform in the block
    const int izs = za + B.lo[2], ize = zb - 1 + B.hi[2];
    load_cells(izs - 1, cells + pmod(izs - 1, 2) * nxc * nyc);
    for (int iz = izs; iz <= ize; ++iz) {
        load_cells(iz, cells + pmod(iz, 2) * nxc * nyc);
        __syncthreads();
        make_nodes(iz, cells + pmod(iz - 1, 2) * nxc * nyc, cells + pmod(iz, 2) * nxc * nyc,
                   nodal + pmod(iz, nzr) * nxn * nyn);
        __syncthreads();
        const int ez = iz - B.hi[2];
        if (ez >= za) out_plane(ez);
    }
}

// y = J' d.  Same grid as the forward kernel.
template <int DIM>
__global__ void __launch_bounds__(kFiltTX * kFiltTY) k_filt_bwd(const double* __restrict__ d, double* __restrict__ y,
                                                               const int* __restrict__ soff,
                                                               const double* __restrict__ sw, int S,
                                                               const double* __restrict__ invW, Dims D, FiltBox B,
                                                               int lz) {
    extern __shared__ double fsm[];
    const int nxc = kFiltTX + 1 + B.hi[0] - B.lo[0], nyc = kFiltTY + 1 + B.hi[1] - B.lo[1];
    const int nxn = kFiltTX + 1, nyn = kFiltTY + 1;
    const int nzr = DIM == 3 ? B.hi[2] - B.lo[2] + 1 : 1;
    double* wd = fsm;                              // [nzr][nyc][nxc]  invW d
    double* nodal = wd + nzr * nxc * nyc;          // [2][nyn][nxn]
    double* w = nodal + 2 * nxn * nyn;             // [S]
    int* off = reinterpret_cast<int*>(w + S);      // [S][3]
    const int tid = threadIdx.x, nth = blockDim.x;
    const int tx = tid % kFiltTX, ty = tid / kFiltTX;
    for (int s = tid; s < S; s += nth) {
        w[s] = sw[s];
        off[3 * s] = soff[3 * s];
        off[3 * s + 1] = soff[3 * s + 1];
        off[3 * s + 2] = soff[3 * s + 2];
    }
    const int ex0 = blockIdx.x * kFiltTX, ey0 = blockIdx.y * kFiltTY;
    const int cx0 = ex0 - B.hi[0], cy0 = ey0 - B.hi[1];   // first cell of the (invW d) window
    const int za = DIM == 3 ? blockIdx.z * lz : 0;
    const int zb = DIM == 3 ? min(za + lz, D.nel[2]) : 1;
    const long long cplane = (long long)D.nel[0] * D.nel[1];
    auto load_wd = [&](int cz, double* dst) {
        const bool zok = DIM == 2 || (cz >= 0 && cz < D.nel[2]);
        for (int ay = ty; ay < nyc; ay += kFiltTY)
            for (int ax = tx; ax < nxc; ax += kFiltTX) {
                const int cx = cx0 + ax, cy = cy0 + ay;
                const bool ok = zok && cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1];
                const long long e = cx + (long long)D.nel[0] * cy + cplane * (DIM == 3 ? cz : 0);
                dst[ay * nxc + ax] = ok ? invW[e] * d[e] : 0.0;
            }
    };
    // node plane iz: valence(n) sum_s w_s (invW d)_{n - off_s}
    auto make_nodes = [&](int iz, double* dst) {
        for (int ay = ty; ay < nyn; ay += kFiltTY)
          for (int ax = tx; ax < nxn; ax += kFiltTX) {
            const int i = ay * nxn + ax;
            const int ix = ex0 + ax, iy = ey0 + ay;
            if (ix >= D.nn[0] || iy >= D.nn[1]) {
                dst[i] = 0.0;
                continue;
            }
            double acc = 0.0;
            for (int s = 0; s < S; ++s) {
                const int cx = ix - off[3 * s], cy = iy - off[3 * s + 1], cz = iz - off[3 * s + 2];
                if (cx < 0 || cx >= D.nel[0] || cy < 0 || cy >= D.nel[1] ||
                    (DIM == 3 && (cz < 0 || cz >= D.nel[2])))
                    continue;
                const double* p = wd + (DIM == 3 ? pmod(cz, nzr) : 0) * nxc * nyc;
                acc += w[s] * p[(cy - cy0) * nxc + (cx - cx0)];
            }
            dst[i] = acc;
          }
    };
    // output cell plane ez from node planes ez (lo) and ez + 1 (hi)
    auto out_plane = [&](int ez, const double* nlo, const double* nhi) {
        {
            const int ax = tx, ay = ty;
            const int ex = ex0 + ax, ey = ey0 + ay;
            if (ex >= D.nel[0] || ey >= D.nel[1]) return;
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < (1 << DIM); ++j) {
                const int bx = j & 1, by = (j >> 1) & 1, bz = (j >> 2) & 1;
                const double* np = bz ? nhi : nlo;
                s += np[(ay + by) * nxn + (ax + bx)];
            }
            y[ex + (long long)D.nel[0] * ey + cplane * ez] = s;
        }
    };
    if (DIM == 2) {
        load_wd(0, wd);
        __syncthreads();
        make_nodes(0, nodal);
        __syncthreads();
        out_plane(0, nodal, nodal);
        return;
    }
    if (za >= zb) return;   // uniform in the block
    // node planes za .. zb; node plane iz reads cell planes iz - hi .. iz - lo
    for (int cz = za - B.hi[2]; cz < za - B.lo[2]; ++cz) load_wd(cz, wd + pmod(cz, nzr) * nxc * nyc);
    for (int iz = za; iz <= zb; ++iz) {
        const int cz = iz - B.lo[2];
        load_wd(cz, wd + pmod(cz, nzr) * nxc * nyc);
        __syncthreads();
        make_nodes(iz, nodal + pmod(iz, 2) * nxn * nyn);
        __syncthreads();
        if (iz > za) out_plane(iz - 1, nodal + pmod(iz - 1, 2) * nxn * nyn, nodal + pmod(iz, 2) * nxn * nyn);
    }
}

}  // namespace tog
