// sm_103a kernels of the SIMP compliance loop (matrix-free operator, Jacobi
// PCG, compliance + sensitivities, node-based filter, OC update).
//
// Reference behaviour restated (TopOpt.jl paths):
//   matvec       src/FEA/matrix_free_operator.jl:66-105   (masked EbE product,
//                fixed dofs y = meandiag * x)
//   PCG          src/FEA/solvers_api.jl:177-220 -> IterativeSolvers cg! with
//                Preconditioners DiagonalPreconditioner
//   compliance   src/Functions/compute_element_energy.jl:18-38, compliance.jl:58-76
//   filters      src/CheqFilters/density_filter.jl:25-121, sens_filter.jl:49-111,
//                CheqFilters.jl:66-118
//   OC           no reference; published optimality-criteria update (88-line code)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "tog_internal.h"
#include "tog_reduce.cuh"
#include "tog_device.cuh"

namespace tog {

// ---------------------------------------------------------------------------
// matrix-free operator, 3D hex8: one element column per thread, marching in z.
// A block owns a 31 x (BY-1) tile of node columns and LZ node planes; the halo
// element row/column/layer is recomputed (deterministic, no atomics).  Node
// contributions are combined across x by warp shuffles, across y through
// shared memory and across z in registers.
// ---------------------------------------------------------------------------
constexpr int MV_BY = 8;
constexpr int MV_LZ = 16;
constexpr int MV2_WARPS = 4;
constexpr int MV2_LY = 32;

template <typename T, int DIM>
struct MvArgs {
    const T* x;            // PLAIN / RESID input (internal layout)
    T* y;                  // PLAIN output; RESID residual output
    const double* f;       // RESID right-hand side
    const T* r;            // PCG residual
    T* P0;                 // PCG search directions (ping-pong by iteration parity)
    T* P1;
    T* q;                  // PCG q = K p
    const T* escale;       // per element E_e
    const T* dinv;         // per node 1 / sum_e E_e
    const uint8_t* fixmask;  // per node bit c = component c prescribed
    T meandiag;
    int nel[3];
    int nn[3];
    PcgState* st;
    double* partials;
    Modal<T, DIM> M;
};

template <typename T, int MODE>
__global__ void __launch_bounds__(32 * MV_BY) k_matvec3(const MvArgs<T, 3> A) {
    __shared__ T xbuf[2][MV_BY][32][2][3];
    const int lane = threadIdx.x, ty = threadIdx.y;
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
    const int nnx = A.nn[0], nny = A.nn[1], nnz = A.nn[2];
    const int ex = 31 * (int)blockIdx.x - 1 + lane;
    const int ey = (MV_BY - 1) * (int)blockIdx.y - 1 + ty;
    const int kz0 = MV_LZ * (int)blockIdx.z;
    const bool own_xy = lane >= 1 && ty >= 1 && ex < nnx && ey < nny;
    const T kd0 = A.M.kdinv[0], kd1 = A.M.kdinv[1], kd2 = A.M.kdinv[2];

    auto load_plane = [&](int kk, T (&v)[3][4]) {
#pragma unroll
        for (int by = 0; by < 2; ++by)
#pragma unroll
            for (int bx = 0; bx < 2; ++bx) {
                const int ix = ex + bx, iy = ey + by;
                const int j = bx + 2 * by;
                v[0][j] = v[1][j] = v[2][j] = T(0);
                if (ix >= 0 && ix < nnx && iy >= 0 && iy < nny && kk >= 0 && kk < nnz) {
                    const long long n = ix + (long long)nnx * (iy + (long long)nny * kk);
                    if (MODE == MV_PCG) {
                        const T d = A.dinv[n];
                        v[0][j] = fma(beta, pold[3 * n + 0], d * kd0 * A.r[3 * n + 0]);
                        v[1][j] = fma(beta, pold[3 * n + 1], d * kd1 * A.r[3 * n + 1]);
                        v[2][j] = fma(beta, pold[3 * n + 2], d * kd2 * A.r[3 * n + 2]);
                    } else {
                        const unsigned m = A.fixmask[n];
                        v[0][j] = (m & 1u) ? T(0) : A.x[3 * n + 0];
                        v[1][j] = (m & 2u) ? T(0) : A.x[3 * n + 1];
                        v[2][j] = (m & 4u) ? T(0) : A.x[3 * n + 2];
                    }
                }
            }
    };

    T lo[3][4], up[3][4];
    load_plane(kz0 - 1, lo);
    T carry[3] = {T(0), T(0), T(0)};
    double acc = 0.0;
    const int kend = min(kz0 + MV_LZ - 1, nelz);
    for (int k = kz0 - 1; k <= kend; ++k) {
        load_plane(k + 1, up);
        T y[3][8];
        const bool inel = ex >= 0 && ex < nelx && ey >= 0 && ey < nely && k >= 0 && k < nelz;
        if (inel) {
            const T rho = A.escale[ex + (long long)nelx * (ey + (long long)nely * k)];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    y[c][j] = lo[c][j];
                    y[c][4 + j] = up[c][j];
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
        // y: row ey+1 contributions move one warp up
        const int par = (k - kz0 + 1) & 1;
#pragma unroll
        for (int bz = 0; bz < 2; ++bz)
#pragma unroll
            for (int c = 0; c < 3; ++c) xbuf[par][ty][lane][bz][c] = col[c][1][bz];
        __syncthreads();
        T row[2][3];
#pragma unroll
        for (int bz = 0; bz < 2; ++bz)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                row[bz][c] = col[c][0][bz] + (ty > 0 ? xbuf[par][ty - 1][lane][bz][c] : T(0));
        // plane k is complete
        if (k >= kz0 && own_xy && k < nnz) {
            const long long n = ex + (long long)nnx * (ey + (long long)nny * k);
            const unsigned m = A.fixmask[n];
            T tot[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) tot[c] = carry[c] + row[0][c];
            if (MODE == MV_PCG) {
                T accf = T(0);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T pv = lo[c][0];
                    const T qv = ((m >> c) & 1u) ? A.meandiag * pv : tot[c];
                    pnew[3 * n + c] = pv;
                    A.q[3 * n + c] = qv;
                    accf = fma(pv, qv, accf);
                }
                acc += (double)accf;
            } else if (MODE == MV_PLAIN) {
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    A.y[3 * n + c] = ((m >> c) & 1u) ? A.meandiag * A.x[3 * n + c] : tot[c];
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T rv = ((m >> c) & 1u) ? T(0) : (T)(A.f[3 * n + c] - (double)tot[c]);
                    A.y[3 * n + c] = rv;
                    acc += (double)rv * (double)rv;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            carry[c] = row[1][c];
#pragma unroll
            for (int j = 0; j < 4; ++j) lo[c][j] = up[c][j];
        }
    }
    if (MODE == MV_PLAIN) return;
    double v[1] = {acc}, tot[1];
    if (grid_reduce_last<1>(v, A.partials, &A.st->cnt[0], tot)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (MODE == MV_PCG) {
                A.st->pq = tot[0];
                if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
                    A.st->status = 4;
                    A.st->done = 1;
                } else {
                    A.st->alpha = A.st->rz / tot[0];
                }
            } else {
                A.st->rr = tot[0];
            }
        }
    }
}

// 2D quad4: one element column (x) per thread, marching in y; warps are
// independent (x tile, y chunk) pieces.  Each warp owns 31 node columns and
// MV2_LY node rows.
template <typename T, int MODE>
__global__ void __launch_bounds__(32 * MV2_WARPS) k_matvec2(const MvArgs<T, 2> A) {
    const int lane = threadIdx.x;
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
    const int nelx = A.nel[0], nely = A.nel[1];
    const int nnx = A.nn[0], nny = A.nn[1];
    const int ex = 31 * (int)blockIdx.x - 1 + lane;
    const int ky0 = MV2_LY * ((int)blockIdx.y * MV2_WARPS + (int)threadIdx.y);
    const bool own_x = lane >= 1 && ex < nnx;
    const T kd0 = A.M.kdinv[0], kd1 = A.M.kdinv[1];

    auto load_row = [&](int kk, T (&v)[2][2]) {
#pragma unroll
        for (int bx = 0; bx < 2; ++bx) {
            const int ix = ex + bx;
            v[0][bx] = v[1][bx] = T(0);
            if (ix >= 0 && ix < nnx && kk >= 0 && kk < nny) {
                const long long n = ix + (long long)nnx * kk;
                if (MODE == MV_PCG) {
                    const T d = A.dinv[n];
                    v[0][bx] = fma(beta, pold[2 * n + 0], d * kd0 * A.r[2 * n + 0]);
                    v[1][bx] = fma(beta, pold[2 * n + 1], d * kd1 * A.r[2 * n + 1]);
                } else {
                    const unsigned m = A.fixmask[n];
                    v[0][bx] = (m & 1u) ? T(0) : A.x[2 * n + 0];
                    v[1][bx] = (m & 2u) ? T(0) : A.x[2 * n + 1];
                }
            }
        }
    };
    T lo[2][2], up[2][2];
    load_row(ky0 - 1, lo);
    T carry[2] = {T(0), T(0)};
    double acc = 0.0;
    const int kend = min(ky0 + MV2_LY - 1, nely);
    for (int k = ky0 - 1; k <= kend; ++k) {
        load_row(k + 1, up);
        T y[2][4];
        const bool inel = ex >= 0 && ex < nelx && k >= 0 && k < nely;
        if (inel) {
            const T rho = A.escale[ex + (long long)nelx * k];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                y[c][0] = lo[c][0];
                y[c][1] = lo[c][1];
                y[c][2] = up[c][0];
                y[c][3] = up[c][1];
            }
            element_apply<T, 2>(A.M, rho, y);
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
            const long long n = ex + (long long)nnx * k;
            const unsigned m = A.fixmask[n];
            T tot[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) tot[c] = carry[c] + col[c][0];
            if (MODE == MV_PCG) {
                T accf = T(0);
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const T pv = lo[c][0];
                    const T qv = ((m >> c) & 1u) ? A.meandiag * pv : tot[c];
                    pnew[2 * n + c] = pv;
                    A.q[2 * n + c] = qv;
                    accf = fma(pv, qv, accf);
                }
                acc += (double)accf;
            } else if (MODE == MV_PLAIN) {
#pragma unroll
                for (int c = 0; c < 2; ++c)
                    A.y[2 * n + c] = ((m >> c) & 1u) ? A.meandiag * A.x[2 * n + c] : tot[c];
            } else {
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const T rv = ((m >> c) & 1u) ? T(0) : (T)(A.f[2 * n + c] - (double)tot[c]);
                    A.y[2 * n + c] = rv;
                    acc += (double)rv * (double)rv;
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
    if (MODE == MV_PLAIN) return;
    double v[1] = {acc}, tot[1];
    if (grid_reduce_last<1>(v, A.partials, &A.st->cnt[0], tot)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (MODE == MV_PCG) {
                A.st->pq = tot[0];
                if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
                    A.st->status = 4;
                    A.st->done = 1;
                } else {
                    A.st->alpha = A.st->rz / tot[0];
                }
            } else {
                A.st->rr = tot[0];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// PCG vector kernels
// ---------------------------------------------------------------------------
template <typename T, int DIM>
__global__ void __launch_bounds__(256) k_pcg_update(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ P0,
                                                    const T* __restrict__ P1, const T* __restrict__ q,
                                                    const T* __restrict__ dinv, const Modal<T, DIM> M,
                                                    long long nnodes, PcgState* st, double* partials,
                                                    const LoopCond cond) {
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) loop_cond_set(cond, false);
        return;
    }
    const int it = st->it;
    const T* __restrict__ p = (it & 1) ? P1 : P0;
    const T alpha = (T)st->alpha;
    T arz = T(0), arr = T(0);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const T d = dinv[n];
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
            const long long i = DIM * n + c;
            x[i] = fma(alpha, p[i], x[i]);
            const T rn = fma(-alpha, q[i], r[i]);
            r[i] = rn;
            arz = fma(rn, d * M.kdinv[c] * rn, arz);
            arr = fma(rn, rn, arr);
        }
    }
    double v[2] = {(double)arz, (double)arr}, tot[2];
    if (grid_reduce_last<2>(v, partials, &st->cnt[1], tot)) {
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

// EnergyCriteria (src/FEA/convergence_criteria.jl:26-45), IterativeSolvers' isconverged
// for it: with xr = x'r and x'Ax = f'x - xr, converged when |x'Ax - E| / x'Ax <= tol and
// |xr| / x'Ax <= tol, E the value of the previous check, which it then replaces; a NaN
// or a negative x'Ax is the reference's DomainError (status 7).  Runs once per completed
// iteration (and once on the start vector), after the update, on FP64 dof arrays.
__global__ void k_energy_init(PcgState* st) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->tol_e = sqrt(fmax(st->tol2, 0.0));   // max(rtol ||r0||, abstol)
        st->tol2 = -1.0;                         // no residual-norm stop
        st->energy = 0.0;
        st->it_e = -1;
        st->done = st->maxit <= 0 ? 1 : 0;
        st->status = st->maxit <= 0 ? 3 : 0;
    }
}

__global__ void __launch_bounds__(256) k_energy_check(const double* __restrict__ x, const double* __restrict__ r,
                                                      const double* __restrict__ f, long long n, PcgState* st,
                                                      double* partials) {
    const int it = st->it;
    if (it == st->it_e || st->status == 7) return;   // nothing new since the last check
    double xr = 0.0, fx = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double xi = x[i];
        xr = fma(xi, r[i], xr);
        fx = fma(f[i], xi, fx);
    }
    double v[2] = {xr, fx}, tot[2];
    if (grid_reduce_last<2>(v, partials, &st->cnt[3], tot)) {
        if (threadIdx.x == 0) {
            const double xAx = tot[1] - tot[0];
            const double dE = xAx - st->energy;
            st->it_e = it;
            if (isnan(dE) || isnan(xAx) || xAx < 0.0) {
                st->status = 7;
                st->done = 1;
            } else {
                const bool conv = fabs(dE) / xAx <= st->tol_e && fabs(tot[0]) / xAx <= st->tol_e;
                st->energy = xAx;
                if (conv && st->status != 4) {
                    st->status = 0;
                    st->done = 1;
                }
            }
        }
    }
}

// Start a PCG solve from the residual already stored in r (x either zeroed here
// or holding the warm start).  tol2 = max(rtol^2 * bnorm2, abstol^2), with
// bnorm2 < 0 meaning "use ||r0||^2".
template <typename T, int DIM>
__global__ void __launch_bounds__(256) k_pcg_init(T* __restrict__ x, const T* __restrict__ r, T* __restrict__ P0,
                                                  T* __restrict__ P1, const T* __restrict__ dinv,
                                                  const Modal<T, DIM> M, long long nnodes, int zero_x, double rtol,
                                                  double abstol, double bnorm2, int maxit, PcgState* st,
                                                  double* partials, double ru_delta2) {
    T arz = T(0), arr = T(0);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const T d = dinv[n];
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
            const long long i = DIM * n + c;
            if (zero_x) x[i] = T(0);
            P0[i] = T(0);
            P1[i] = T(0);
            const T rn = r[i];
            arz = fma(rn, d * M.kdinv[c] * rn, arz);
            arr = fma(rn, rn, arr);
        }
    }
    double v[2] = {(double)arz, (double)arr}, tot[2];
    if (grid_reduce_last<2>(v, partials, &st->cnt[1], tot)) {
        if (threadIdx.x == 0) {
            st->rz = tot[0];
            st->rz_old = 0.0;
            st->beta = 0.0;
            st->alpha = 0.0;
            st->rr = tot[1];
            st->rr0 = tot[1];
            const double b2 = bnorm2 >= 0.0 ? bnorm2 : tot[1];
            st->tol2 = fmax(rtol * rtol * b2, abstol * abstol);
            st->it = 0;
            st->maxit = maxit;
            st->status = 0;
            st->done = (tot[1] <= st->tol2 || maxit <= 0) ? 1 : 0;
            if (maxit <= 0 && tot[1] > st->tol2) st->status = 3;
            st->pq = 0.0;
            st->rr_max = tot[1];
            st->ru_delta2 = ru_delta2;
        }
    }
}

// FP32 inner solve of the iterative refinement: r32 = r64 / ||r64||
template <int DIM>
__global__ void __launch_bounds__(256) k_ir_scale(const double* __restrict__ r64, float* __restrict__ r32,
                                                  long long ndofs, const PcgState* st64) {
    const double s = st64->rr > 0.0 ? 1.0 / sqrt(st64->rr) : 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndofs;
         i += (long long)gridDim.x * blockDim.x)
        r32[i] = (float)(r64[i] * s);
}
// u64 += s * x32
__global__ void __launch_bounds__(256) k_ir_correct(double* __restrict__ u, const float* __restrict__ x32,
                                                    long long ndofs, double s) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndofs;
         i += (long long)gridDim.x * blockDim.x)
        u[i] = fma(s, (double)x32[i], u[i]);
}

// Reliable update of the FP32 PCG: r32 = r64 / s_new (the FP64 true residual),
// x32 = 0, the last direction rescaled by s_old / s_new, and the PCG scalars
// recomputed so that the next direction is z + beta p with the same p.
template <int DIM>
__global__ void __launch_bounds__(256) k_ru_rescale(const double* __restrict__ r64, float* __restrict__ r32,
                                                    float* __restrict__ x32, float* __restrict__ P0,
                                                    float* __restrict__ P1, const float* __restrict__ dinv,
                                                    const Modal<float, DIM> M, long long nnodes, double s_old,
                                                    double s_new, double tol2, PcgState* st, double* partials) {
    const int it = st->it;                      // the last direction is P[(it - 1) & 1]
    float* __restrict__ p = ((it - 1) & 1) ? P1 : P0;
    const double inv = 1.0 / s_new;
    const float ratio = (float)(s_old / s_new);
    float arz = 0.f, arr = 0.f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const float d = dinv[n];
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
            const long long i = DIM * n + c;
            const float rn = (float)(r64[i] * inv);
            r32[i] = rn;
            x32[i] = 0.f;
            p[i] *= ratio;
            arz = fmaf(rn, d * M.kdinv[c] * rn, arz);
            arr = fmaf(rn, rn, arr);
        }
    }
    double v[2] = {(double)arz, (double)arr}, tot[2];
    if (grid_reduce_last<2>(v, partials, &st->cnt[1], tot)) {
        if (threadIdx.x == 0) {
            const double rz_prev = st->rz_old * (s_old / s_new) * (s_old / s_new);
            st->rz = tot[0];
            st->beta = rz_prev > 0.0 ? tot[0] / rz_prev : 0.0;
            st->rr = tot[1];
            st->rr_max = tot[1];
            st->tol2 = tol2;
            st->status = 0;
            st->done = (tot[1] <= tol2) ? 1 : 0;
        }
    }
}

// ---------------------------------------------------------------------------
// densities -> element scales and the Jacobi diagonal
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_escale(const double* __restrict__ vars, double* __restrict__ e64,
                                                float* __restrict__ e32, long long ncells, double xmin, double p,
                                                int ip) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncells;
         e += (long long)gridDim.x * blockDim.x) {
        const double v = fma(ipow(vars[e], p, ip), 1.0 - xmin, xmin);
        e64[e] = v;
        e32[e] = (float)v;
    }
}

template <int DIM>
__global__ void __launch_bounds__(256) k_nodesum(const double* __restrict__ e64, double* __restrict__ d64,
                                                 float* __restrict__ d32, Dims D) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < D.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(n % D.nn[0]);
        const long long t = n / D.nn[0];
        const int iy = (int)(t % D.nn[1]);
        const int iz = DIM == 3 ? (int)(t / D.nn[1]) : 0;
        double s = 0.0;
#pragma unroll
        for (int bz = 0; bz < (DIM == 3 ? 2 : 1); ++bz)
#pragma unroll
            for (int by = 0; by < 2; ++by)
#pragma unroll
                for (int bx = 0; bx < 2; ++bx) {
                    const int cx = ix - 1 + bx, cy = iy - 1 + by, cz = DIM == 3 ? iz - 1 + bz : 0;
                    if (cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1] && (DIM == 2 || (cz >= 0 && cz < D.nel[2])))
                        s += e64[cx + (long long)D.nel[0] * (cy + (long long)D.nel[1] * cz)];
                }
        const double iv = s > 0.0 ? 1.0 / s : 0.0;
        d64[n] = iv;
        d32[n] = (float)iv;
    }
}

// ---------------------------------------------------------------------------
// compliance + sensitivities (FP64): ce_e = u_e' Ke u_e, c = sum rho_e ce_e,
// grad_e = -drho_e ce_e
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(256) k_compliance(const double* __restrict__ u, const double* __restrict__ vars,
                                                    const Modal<double, DIM> M, double xmin, double p, int ip,
                                                    Dims D, double* __restrict__ grad, double* __restrict__ cell_ce,
                                                    double* partials, unsigned* counter, double* result) {
    constexpr int NC = 1 << DIM;
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < D.ncells;
         e += (long long)gridDim.x * blockDim.x) {
        const int ex = (int)(e % D.nel[0]);
        const long long t = e / D.nel[0];
        const int ey = (int)(t % D.nel[1]);
        const int ez = DIM == 3 ? (int)(t / D.nel[1]) : 0;
        double uc[DIM][NC];
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            const int bx = j & 1, by = (j >> 1) & 1, bz = (j >> 2) & 1;
            const long long n = (ex + bx) + (long long)D.nn[0] * ((ey + by) + (long long)D.nn[1] * (ez + bz));
#pragma unroll
            for (int c = 0; c < DIM; ++c) uc[c][j] = u[DIM * n + c];
        }
        const double ce = element_energy<DIM>(M, uc);
        const double x = vars[e];
        const double rho = fma(ipow(x, p, ip), 1.0 - xmin, xmin);
        const double drho = (1.0 - xmin) * p * (p == 0.0 ? 0.0 : ipow(x, p - 1.0, ip > 0 ? ip - 1 : -1));
        grad[e] = -drho * ce;
        if (cell_ce) cell_ce[e] = ce;
        acc = fma(rho, ce, acc);
    }
    double v[1] = {acc}, tot[1];
    if (grid_reduce_last<1>(v, partials, counter, tot))
        if (threadIdx.x == 0) *result = tot[0];
}

// ---------------------------------------------------------------------------
// node-based filter (FP64).  M1: element -> node average over the node's
// cells; M2: node -> element cone with weight (rmin - d) * valence(node).
// J = M2 M1 (DensityFilterFun forward, SensFilterFun pullback); J' = M1' M2'.
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(256) k_filt_node_avg(const double* __restrict__ xe, double* __restrict__ nodal,
                                                       Dims D) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < D.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(n % D.nn[0]);
        const long long t = n / D.nn[0];
        const int iy = (int)(t % D.nn[1]);
        const int iz = DIM == 3 ? (int)(t / D.nn[1]) : 0;
        double s = 0.0;
        int cnt = 0;
#pragma unroll
        for (int bz = 0; bz < (DIM == 3 ? 2 : 1); ++bz)
#pragma unroll
            for (int by = 0; by < 2; ++by)
#pragma unroll
                for (int bx = 0; bx < 2; ++bx) {
                    const int cx = ix - 1 + bx, cy = iy - 1 + by, cz = DIM == 3 ? iz - 1 + bz : 0;
                    if (cx >= 0 && cx < D.nel[0] && cy >= 0 && cy < D.nel[1] && (DIM == 2 || (cz >= 0 && cz < D.nel[2]))) {
                        s += xe[cx + (long long)D.nel[0] * (cy + (long long)D.nel[1] * cz)];
                        ++cnt;
                    }
                }
        nodal[n] = cnt ? s / cnt : 0.0;
    }
}

// out_e = sum_{n in e} nodal_n / count_n   (M1')
template <int DIM>
__global__ void __launch_bounds__(256) k_filt_node_avg_T(const double* __restrict__ nodal, double* __restrict__ out,
                                                         Dims D) {
    constexpr int NC = 1 << DIM;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < D.ncells;
         e += (long long)gridDim.x * blockDim.x) {
        const int ex = (int)(e % D.nel[0]);
        const long long t = e / D.nel[0];
        const int ey = (int)(t % D.nel[1]);
        const int ez = DIM == 3 ? (int)(t / D.nel[1]) : 0;
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            const int ix = ex + (j & 1), iy = ey + ((j >> 1) & 1), iz = ez + ((j >> 2) & 1);
            const long long n = ix + (long long)D.nn[0] * (iy + (long long)D.nn[1] * iz);
            s += nodal[n] / valence<DIM>(ix, iy, iz, D);
        }
        out[e] = s;
    }
}

// stencil entry s: node offset (dx, dy, dz) from the element's lower corner, weight w
template <int DIM>
__global__ void __launch_bounds__(256) k_filt_invW(const int* __restrict__ soff, const double* __restrict__ sw,
                                                   int S, double* __restrict__ invW, Dims D) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < D.ncells;
         e += (long long)gridDim.x * blockDim.x) {
        const int ex = (int)(e % D.nel[0]);
        const long long t = e / D.nel[0];
        const int ey = (int)(t % D.nel[1]);
        const int ez = DIM == 3 ? (int)(t / D.nel[1]) : 0;
        double W = 0.0;
        for (int s = 0; s < S; ++s) {
            const int ix = ex + soff[3 * s], iy = ey + soff[3 * s + 1], iz = ez + soff[3 * s + 2];
            if (ix >= 0 && ix < D.nn[0] && iy >= 0 && iy < D.nn[1] && (DIM == 2 || (iz >= 0 && iz < D.nn[2])))
                W += sw[s] * valence<DIM>(ix, iy, iz, D);
        }
        invW[e] = W > 0.0 ? 1.0 / W : 0.0;
    }
}

// y_e = invW_e * sum_s w_s valence(n) nodal_n   (M2)
template <int DIM>
__global__ void __launch_bounds__(256) k_filt_cone(const double* __restrict__ nodal, double* __restrict__ ye,
                                                   const int* __restrict__ soff, const double* __restrict__ sw, int S,
                                                   const double* __restrict__ invW, const double* __restrict__ xin,
                                                   Dims D) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < D.ncells;
         e += (long long)gridDim.x * blockDim.x) {
        const int ex = (int)(e % D.nel[0]);
        const long long t = e / D.nel[0];
        const int ey = (int)(t % D.nel[1]);
        const int ez = DIM == 3 ? (int)(t / D.nel[1]) : 0;
        double s_ = 0.0;
        for (int s = 0; s < S; ++s) {
            const int ix = ex + soff[3 * s], iy = ey + soff[3 * s + 1], iz = ez + soff[3 * s + 2];
            if (ix >= 0 && ix < D.nn[0] && iy >= 0 && iy < D.nn[1] && (DIM == 2 || (iz >= 0 && iz < D.nn[2]))) {
                const long long n = ix + (long long)D.nn[0] * (iy + (long long)D.nn[1] * iz);
                s_ += sw[s] * valence<DIM>(ix, iy, iz, D) * nodal[n];
            }
        }
        // an element with no node inside rmin keeps its input (reference skips the row)
        ye[e] = invW[e] > 0.0 ? s_ * invW[e] : (xin ? xin[e] : 0.0);
    }
}

// nodal_n = valence(n) * sum_s w_s invW_e d_e over e = n - off_s   (M2')
template <int DIM>
__global__ void __launch_bounds__(256) k_filt_cone_T(const double* __restrict__ de, double* __restrict__ nodal,
                                                     const int* __restrict__ soff, const double* __restrict__ sw,
                                                     int S, const double* __restrict__ invW, Dims D) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < D.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(n % D.nn[0]);
        const long long t = n / D.nn[0];
        const int iy = (int)(t % D.nn[1]);
        const int iz = DIM == 3 ? (int)(t / D.nn[1]) : 0;
        double s_ = 0.0;
        for (int s = 0; s < S; ++s) {
            const int ex = ix - soff[3 * s], ey = iy - soff[3 * s + 1], ez = iz - soff[3 * s + 2];
            if (ex >= 0 && ex < D.nel[0] && ey >= 0 && ey < D.nel[1] && (DIM == 2 || (ez >= 0 && ez < D.nel[2]))) {
                const long long e = ex + (long long)D.nel[0] * (ey + (long long)D.nel[1] * ez);
                s_ += sw[s] * invW[e] * de[e];
            }
        }
        nodal[n] = s_ * valence<DIM>(ix, iy, iz, D);
    }
}

// ---------------------------------------------------------------------------
// OC update (FP64).  B_e = x_e sqrt(max(0,-dc_e)/dv_e); bisection on lambda
// with x_new = clamp(B_e / sqrt(lambda), max(0,x-move), min(1,x+move)).
// fpos (optional) is the active-element mask: fpos[e] < 0 pins cell e (-1 black at
// density 1, -2 white at density 0) by collapsing its bounds onto that value.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double oc_new(double xe, double b, double move, const int* __restrict__ fpos,
                                         long long e) {
    double lo = fmax(0.0, xe - move), hi = fmin(1.0, xe + move);
    if (fpos) {
        const int p = fpos[e];
        if (p < 0) lo = hi = (p == -1) ? 1.0 : 0.0;
    }
    return fmin(hi, fmax(lo, b));
}
__global__ void __launch_bounds__(256) k_oc_prep(const double* __restrict__ x, const double* __restrict__ dc,
                                                 const double* __restrict__ dv, double* __restrict__ B, long long n,
                                                 OcState* oc, double l1, double l2, double tol, double target,
                                                 double move, int maxsteps) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        B[e] = x[e] * sqrt(fmax(0.0, -dc[e]) / dv[e]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        oc->l1 = l1;
        oc->l2 = l2;
        oc->tol = tol;
        oc->target = target;
        oc->move = move;
        oc->steps = 0;
        oc->maxsteps = maxsteps;
        oc->done = ((l2 - l1) / (l1 + l2) <= tol) ? 1 : 0;
        oc->vol = 0.0;
        oc->change = 0.0;
    }
}

__global__ void __launch_bounds__(256) k_oc_step(const double* __restrict__ x, const double* __restrict__ B,
                                                 const double* __restrict__ w, long long n, OcState* oc,
                                                 double* partials, const int* __restrict__ fpos,
                                                 const LoopCond cond) {
    if (oc->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) loop_cond_set(cond, false);
        return;
    }
    const double lmid = 0.5 * (oc->l2 + oc->l1);
    const double s = 1.0 / sqrt(lmid);
    const double move = oc->move;
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const double xn = oc_new(x[e], B[e] * s, move, fpos, e);
        acc = fma(w[e], xn, acc);
    }
    double v[1] = {acc}, tot[1];
    if (grid_reduce_last<1>(v, partials, &oc->cnt[0], tot)) {
        if (threadIdx.x == 0) {
            oc->vol = tot[0];
            if (tot[0] > oc->target)
                oc->l1 = lmid;
            else
                oc->l2 = lmid;
            oc->steps += 1;
            if ((oc->l2 - oc->l1) / (oc->l1 + oc->l2) <= oc->tol || oc->steps >= oc->maxsteps) oc->done = 1;
            loop_cond_set(cond, !oc->done);
        }
    }
}

// Sets a WHILE node's condition from an OC state (the bisection runs unless it is done).
__global__ void k_oc_cond_init(const OcState* __restrict__ oc, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0) cudaGraphSetConditional(h, oc->done ? 0u : 1u);
}

__global__ void __launch_bounds__(256) k_oc_final(const double* __restrict__ x, const double* __restrict__ B,
                                                  double* __restrict__ xnew, long long n, OcState* oc,
                                                  double* partials, const double* __restrict__ w,
                                                  const int* __restrict__ fpos) {
    const double lmid = 0.5 * (oc->l2 + oc->l1);
    const double s = 1.0 / sqrt(lmid);
    const double move = oc->move;
    double mx = 0.0, vol = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const double xe = x[e];
        const double xn = oc_new(xe, B[e] * s, move, fpos, e);
        xnew[e] = xn;
        mx = fmax(mx, fabs(xn - xe));
        vol = fma(w[e], xn, vol);
    }
    double v[1] = {mx}, tot[1];
    if (grid_reduce_last<1, true>(v, partials, &oc->cnt[1], tot)) {
        if (threadIdx.x == 0) {
            oc->change = tot[0];
            oc->lmid = lmid;
        }
    }
    double v2[1] = {vol}, tot2[1];
    if (grid_reduce_last<1>(v2, partials + 2 * gridDim.x, &oc->cnt[2], tot2)) {
        if (threadIdx.x == 0) oc->vol = tot2[0];
    }
}

// ---------------------------------------------------------------------------
// FixedElementProjectorFun (src/Functions/fixed_element.jl:44-79) on the device.
// fpos[e] >= 0 is the position of free cell e in x_free (free cells in cell order),
// -1 a black cell (density 1), -2 a white cell (density 0).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fixed_project(const double* __restrict__ xf, const int* __restrict__ fpos,
                                                       double* __restrict__ rho, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int p = fpos[e];
        rho[e] = p >= 0 ? xf[p] : (p == -1 ? 1.0 : 0.0);
    }
}
// pullback: the cotangent of the free cells, in x_free order (fixed cells receive none)
__global__ void __launch_bounds__(256) k_fixed_pullback(const double* __restrict__ drho,
                                                        const int* __restrict__ fpos, double* __restrict__ dxf,
                                                        long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int p = fpos[e];
        if (p >= 0) dxf[p] = drho[e];
    }
}
// hold the fixed cells of a full design vector at their densities
__global__ void __launch_bounds__(256) k_fixed_pin(double* __restrict__ x, const int* __restrict__ fpos, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int p = fpos[e];
        if (p < 0) x[e] = (p == -1) ? 1.0 : 0.0;
    }
}

// FP64 -> FP32 copy of a dof vector
__global__ void __launch_bounds__(256) k_cast_f32(const double* __restrict__ src, float* __restrict__ dst,
                                                  long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

// Output of one PCG operator launch in FP64: p, and q with the prescribed rows
// replaced by meandiag p (what the PCG update does with them)
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_operator_out(const T* __restrict__ p, const T* __restrict__ q,
                                                          const uint8_t* __restrict__ fixmask, double meandiag,
                                                          long long nnodes, int dim, double* __restrict__ pout,
                                                          double* __restrict__ qout) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const unsigned m = fixmask[n];
        for (int c = 0; c < dim; ++c) {
            const long long i = dim * n + c;
            const double pv = (double)p[i];
            pout[i] = pv;
            qout[i] = ((m >> c) & 1u) ? meandiag * pv : (double)q[i];
        }
    }
}

// ---------------------------------------------------------------------------
// dof permutation between the reference (Ferrite) order and the internal order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gather_d(const double* __restrict__ src, const int* __restrict__ idx,
                                                  double* __restrict__ dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

}  // namespace tog
