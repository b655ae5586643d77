// MMA, the method of moving asymptotes (Svanberg 1987), for one inequality
// constraint on the device: the optimizer TopOpt.jl's SIMP examples call through
// Nonconvex (MMA87, e.g. docs/tutorials/simp.qmd:107-114,
// test/integration/test_end_to_end.jl:30-47).  Nonconvex's MMA is not part of
// TopOpt.jl, so this restates the published method, in the form of Svanberg's
// "MMA and GCMMA" notes (2007): asymptotes from the last two iterates (init 0.5,
// increase 1.2, decrease 0.7, kept within [0.01, 10] design ranges of x), bounds
// alpha / beta with albefa 0.1 and move 0.5, the approximation coefficients
// p = (U-x)^2 (max(df,0) + 1e-3 |df| + 1e-5), q = (x-L)^2 (max(-df,0) + 1e-3 |df| + 1e-5)
// (design range 1), and the subproblem solved through its dual in the one
// multiplier lambda: x_j(lambda) minimises (p0 + lambda p1)/(U-x) + (q0 + lambda q1)/(x-L)
// on [alpha, beta] in closed form, and lambda makes the approximated constraint
// active (bisection in log lambda on [1e-30, 1e30]; lambda = 0 when it is inactive).
//
// Kernels: k_mma_prep (asymptotes, bounds, coefficients, right-hand side),
// kMmaMaxSteps of k_mma_step (one dual evaluation and bisection step each, a
// graph), k_mma_final (new design, change, iterate history).  All FP64, grid-stride,
// deterministic reductions.
#pragma once
#include <cuda_runtime.h>

#include "tog_reduce.cuh"

namespace tog {

constexpr int kMmaMaxSteps = 72;   // 1 evaluation at lambda = 0, then bisection in log lambda

struct MmaState {
    double lo, hi;    // bracket of log(lambda)
    double lam;       // the multiplier (final once done)
    double r;         // right-hand side: sum(p1/(U-x) + q1/(x-L)) - g
    double g;         // constraint value at x
    double change;    // max |x_new - x|
    double vol;       // sum(w x_new) (when volume weights are given)
    double tol;       // stop when hi - lo <= tol
    int steps, done, maxsteps, use_w;   // use_w: volume weights given (g and vol from them)
    unsigned cnt[4];
};

struct MmaArgs {
    const double* x;
    const double* df0;   // objective gradient
    const double* dg;    // constraint gradient
    const double* w;     // volume weights: g = sum(w x) - volfrac when set
    const int* fpos;     // active-element mask (optional): < 0 pins the cell
    double *low, *upp, *xold1, *xold2;   // asymptotes and iterate history (persist)
    double *alfa, *beta, *p0, *q0, *p1, *q1;
    double* xnew;
    long long n;
    MmaState* st;
    double* partials;
};

__device__ __forceinline__ double mma_x(double P, double Q, double L, double U, double a, double b) {
    const double sp = sqrt(P), sq = sqrt(Q);
    const double xe = (L * sp + U * sq) / (sp + sq);
    return fmin(b, fmax(a, xe));
}

// k is the 1-based MMA iteration; g the constraint value (ignored when A.w is set).
__global__ void __launch_bounds__(256) k_mma_prep(const MmaArgs A, int k, double g, double volfrac, double move) {
    constexpr double asyinit = 0.5, asyincr = 1.2, asydecr = 0.7, albefa = 0.1, raa = 1e-5;
    double sr = 0.0, sv = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < A.n;
         e += (long long)gridDim.x * blockDim.x) {
        const double x = A.x[e];
        double L, U;
        if (k <= 2) {
            L = x - asyinit;
            U = x + asyinit;
        } else {
            const double x1 = A.xold1[e], x2 = A.xold2[e];
            const double zz = (x - x1) * (x1 - x2);
            const double f = zz > 0.0 ? asyincr : (zz < 0.0 ? asydecr : 1.0);
            L = x - f * (x1 - A.low[e]);
            U = x + f * (A.upp[e] - x1);
            L = fmin(fmax(L, x - 10.0), x - 0.01);
            U = fmin(fmax(U, x + 0.01), x + 10.0);
        }
        double a = fmax(fmax(L + albefa * (x - L), x - move), 0.0);
        double b = fmin(fmin(U - albefa * (U - x), x + move), 1.0);
        if (A.fpos) {
            const int p = A.fpos[e];
            if (p < 0) a = b = (p == -1) ? 1.0 : 0.0;
        }
        const double ux2 = (U - x) * (U - x), xl2 = (x - L) * (x - L);
        const double d0 = A.df0[e], d1 = A.dg[e];
        const double r0 = 1e-3 * fabs(d0) + raa, r1 = 1e-3 * fabs(d1) + raa;
        const double p1 = (fmax(d1, 0.0) + r1) * ux2, q1 = (fmax(-d1, 0.0) + r1) * xl2;
        A.low[e] = L;
        A.upp[e] = U;
        A.alfa[e] = a;
        A.beta[e] = b;
        A.p0[e] = (fmax(d0, 0.0) + r0) * ux2;
        A.q0[e] = (fmax(-d0, 0.0) + r0) * xl2;
        A.p1[e] = p1;
        A.q1[e] = q1;
        sr += p1 / (U - x) + q1 / (x - L);
        if (A.w) sv = fma(A.w[e], x, sv);
    }
    double v[2] = {sr, sv}, tot[2];
    if (grid_reduce_last<2>(v, A.partials, &A.st->cnt[0], tot)) {
        if (threadIdx.x == 0) {
            MmaState* s = A.st;
            s->g = A.w ? tot[1] - volfrac : g;
            s->r = tot[0] - s->g;
            s->lo = log(1e-30);
            s->hi = log(1e30);
            s->lam = 0.0;
            s->tol = 1e-12;
            s->steps = 0;
            s->done = 0;
            s->maxsteps = kMmaMaxSteps;
            s->change = 0.0;
            s->vol = 0.0;
            s->use_w = A.w ? 1 : 0;
        }
    }
}

__global__ void __launch_bounds__(256) k_mma_step(const MmaArgs A) {
    MmaState* s = A.st;
    if (s->done) return;
    const int steps = s->steps;
    const double lam = steps == 0 ? 0.0 : exp(0.5 * (s->lo + s->hi));
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < A.n;
         e += (long long)gridDim.x * blockDim.x) {
        const double L = A.low[e], U = A.upp[e], p1 = A.p1[e], q1 = A.q1[e];
        const double xe = mma_x(fma(lam, p1, A.p0[e]), fma(lam, q1, A.q0[e]), L, U, A.alfa[e], A.beta[e]);
        acc += p1 / (U - xe) + q1 / (xe - L);
    }
    double v[1] = {acc}, tot[1];
    if (grid_reduce_last<1>(v, A.partials, &s->cnt[1], tot)) {
        if (threadIdx.x == 0) {
            const double h = tot[0] - s->r;   // dual gradient: approximated constraint at x(lambda)
            if (steps == 0) {
                if (h <= 0.0) {               // inactive at lambda = 0
                    s->lam = 0.0;
                    s->done = 1;
                }
            } else {
                const double mid = 0.5 * (s->lo + s->hi);
                if (h > 0.0)
                    s->lo = mid;   // constraint violated: larger multiplier
                else
                    s->hi = mid;
            }
            s->steps = steps + 1;
            if (!s->done && (s->hi - s->lo <= s->tol || s->steps >= s->maxsteps)) {
                s->lam = exp(0.5 * (s->lo + s->hi));
                s->done = 1;
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_mma_final(const MmaArgs A) {
    MmaState* s = A.st;
    const double lam = s->lam;
    const bool use_w = s->use_w && A.w;
    double mx = 0.0, vol = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < A.n;
         e += (long long)gridDim.x * blockDim.x) {
        const double x = A.x[e];
        const double xn = mma_x(fma(lam, A.p1[e], A.p0[e]), fma(lam, A.q1[e], A.q0[e]), A.low[e], A.upp[e],
                                A.alfa[e], A.beta[e]);
        A.xnew[e] = xn;
        A.xold2[e] = A.xold1[e];
        A.xold1[e] = x;
        mx = fmax(mx, fabs(xn - x));
        if (use_w) vol = fma(A.w[e], xn, vol);
    }
    double v[1] = {mx}, tot[1];
    if (grid_reduce_last<1, true>(v, A.partials, &s->cnt[2], tot))
        if (threadIdx.x == 0) s->change = tot[0];
    double v2[1] = {vol}, tot2[1];
    if (grid_reduce_last<1>(v2, A.partials + 2 * gridDim.x, &s->cnt[3], tot2))
        if (threadIdx.x == 0) s->vol = tot2[0];
}

}  // namespace tog
