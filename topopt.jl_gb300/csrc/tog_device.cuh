// Device-side building blocks shared by the kernels of libtopopt_gb300: the
// modal (Hadamard-transformed) element operator, the penalty power and the node
// valence of a structured grid.
#pragma once
#include <cuda_runtime.h>
#include "tog_internal.h"

namespace tog {

// ---------------------------------------------------------------------------
// modal element operator
// ---------------------------------------------------------------------------
template <typename T, int NC>
__device__ __forceinline__ void hadamard_fwd(T (&v)[NC]) {
#pragma unroll
    for (int s = 1; s < NC; s <<= 1)
#pragma unroll
        for (int i = 0; i < NC; ++i)
            if (!(i & s)) {
                T a = v[i], b = v[i + s];
                v[i] = a + b;
                v[i + s] = b - a;
            }
}
template <typename T, int NC>
__device__ __forceinline__ void hadamard_inv(T (&v)[NC]) {
#pragma unroll
    for (int s = NC >> 1; s > 0; s >>= 1)
#pragma unroll
        for (int i = 0; i < NC; ++i)
            if (!(i & s)) {
                T a = v[i], b = v[i + s];
                v[i] = a - b;
                v[i + s] = a + b;
            }
}

// b = rho * M a   (a, b in modal space; b[.][0] = 0)
template <typename T, int DIM>
__device__ __forceinline__ void modal_mul(const Modal<T, DIM>& M, T rho, const T (&a)[DIM][1 << DIM],
                                          T (&b)[DIM][1 << DIM]) {
    constexpr int NC = 1 << DIM;
#pragma unroll
    for (int c = 0; c < DIM; ++c) b[c][0] = T(0);
#pragma unroll
    for (int m = 1; m < NC; ++m)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
            T acc = M.D[m][c] * a[c][m];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                if (d != c && (((m >> c) & 1) != ((m >> d) & 1)))
                    acc = fma(M.O[m][c][d], a[d][m ^ (1 << c) ^ (1 << d)], acc);
            b[c][m] = rho * acc;
        }
}

// u[c][corner] -> y[c][corner] = rho * Ke u
template <typename T, int DIM>
__device__ __forceinline__ void element_apply(const Modal<T, DIM>& M, T rho, T (&u)[DIM][1 << DIM]) {
    constexpr int NC = 1 << DIM;
#pragma unroll
    for (int c = 0; c < DIM; ++c) hadamard_fwd<T, NC>(u[c]);
    T b[DIM][NC];
    modal_mul<T, DIM>(M, rho, u, b);
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
        hadamard_inv<T, NC>(b[c]);
#pragma unroll
        for (int n = 0; n < NC; ++n) u[c][n] = b[c][n];
    }
}

// u_e' Ke u_e from corner values (FP64)
template <int DIM>
__device__ __forceinline__ double element_energy(const Modal<double, DIM>& M, double (&u)[DIM][1 << DIM]) {
    constexpr int NC = 1 << DIM;
#pragma unroll
    for (int c = 0; c < DIM; ++c) hadamard_fwd<double, NC>(u[c]);
    double b[DIM][NC];
    modal_mul<double, DIM>(M, 1.0, u, b);
    double e = 0.0;
#pragma unroll
    for (int c = 0; c < DIM; ++c)
#pragma unroll
        for (int m = 1; m < NC; ++m) e = fma(u[c][m], b[c][m], e);
    return e;
}

__device__ __forceinline__ double ipow(double x, double p, int ip) {
    if (ip >= 0) {
        double r = 1.0;
        for (int i = 0; i < ip; ++i) r *= x;
        return r;
    }
    return pow(x, p);
}

template <int DIM>
__device__ __forceinline__ int valence(int ix, int iy, int iz, const Dims& D) {
    int v = (ix > 0 && ix < D.nel[0] ? 2 : 1) * (iy > 0 && iy < D.nel[1] ? 2 : 1);
    if (DIM == 3) v *= (iz > 0 && iz < D.nel[2] ? 2 : 1);
    return v;
}

}  // namespace tog
