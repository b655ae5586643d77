// Internal definitions shared by the host code and the sm_103a kernels of
// libtopopt_gb300.  Nothing here is part of the C ABI (see include/topopt_gb300.h).
//
// Data layout in HBM (all arrays owned by one tog_handle):
//   * nodes are numbered lexicographically, x fastest: n = ix + nnx*(iy + nny*iz);
//     a nodal vector stores its `dim` components interleaved (AoS): v[dim*n + c].
//     The reference (Ferrite first-touch) dof order is applied only at the
//     C-ABI boundary through a dof permutation.
//   * elements are numbered x fastest, exactly as the reference's cells, so
//     element arrays (densities, sensitivities) cross the boundary unpermuted.
//   * the element stiffness is stored in a modal basis: a = T u_e with T the
//     2x2(x2) Hadamard transform of the element's corner values, Ke = T' M T.
//     For a rectangular element with isotropic material M has 45 (3D) / 10 (2D)
//     non-zeros instead of 576 / 64, which is what makes the matrix-free
//     operator affordable on CUDA cores.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tog {

// Corner index inside an element: n = bx + 2*by (+ 4*bz).  Ferrite's local
// node order (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1)
// maps to corner n via kFerriteToCorner.
static constexpr int kFerriteToCorner[8] = {0, 1, 3, 2, 4, 5, 7, 6};

// Modal element operator: y_mode(m,c) = D[m][c] a(m,c) + sum_{d != c, bit_c(m) != bit_d(m)}
// O[m][c][d] a(m ^ (1<<c) ^ (1<<d), d).  Mode 0 (rigid translation) is zero.
template <typename T, int DIM>
struct Modal {
    T D[1 << DIM][DIM];
    T O[1 << DIM][DIM][DIM];
    T kdinv[DIM];   // 1 / Ke(a,a) for component c (identical at every corner)
};

// Condition of a conditional WHILE graph node that runs a loop on the device (the PCG
// iterations, the OC bisection): the loop's last kernel sets it to "continue" while the
// state is not done.  `on` is 0 for launches outside such a graph.
struct LoopCond {
    cudaGraphConditionalHandle h;
    int on;
};
#ifdef __CUDACC__
__device__ __forceinline__ void loop_cond_set(const LoopCond& c, bool go) {
    if (c.on) cudaGraphSetConditional(c.h, go ? 1u : 0u);
}
#endif

// Modes of the matrix-free operator kernels: y = K x, the fused PCG direction
// update + K p + p.q, and the FP64 residual f - K x.
enum { MV_PLAIN = 0, MV_PCG = 1, MV_RESID = 2 };

// Solver state kept in device memory so that a whole PCG iteration runs
// without a host round trip.  Written only by the "last block" of a kernel.
struct PcgState {
    double rz;       // r . z of the current iterate
    double rz_old;
    double alpha;
    double beta;
    double rr;       // ||r||^2
    double rr0;      // ||r_0||^2
    double tol2;     // stop when rr <= tol2
    double pq;
    int it;          // completed iterations
    int done;        // 1 = stop (converged, breakdown or maxit)
    int maxit;
    int status;      // 0 running/converged, 3 = not converged at maxit, 4 = breakdown,
                     // 6 = paused for a reliable update, 7 = EnergyCriteria domain error
    unsigned cnt[4]; // last-block counters
    double rr_max;   // largest ||r||^2 since the last reliable update
    double ru_delta2;// pause when ||r||^2 < ru_delta2 * rr_max (0 = never)
    // EnergyCriteria (FP64 solves): x'Ax at the last check, its tolerance, the iteration
    // the last check saw
    double energy;
    double tol_e;
    int it_e;
    int pad_e;
};

struct OcState {
    double l1, l2, tol, target, move;
    double vol, change, lmid;
    int steps, done, maxsteps, pad;
    unsigned cnt[4];
};

struct Dims {
    int dim;
    int nel[3];
    int nn[3];
    long long nnodes, ncells;
};

// Records the message returned by tog_last_error() and returns code.
int set_error(int code, const char* msg);

}  // namespace tog
