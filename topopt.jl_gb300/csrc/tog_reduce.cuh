// Deterministic grid reductions shared by the kernels of libtopopt_gb300:
// per-block partial sums, then the last block to finish (threadfence + atomic
// counter, no spin-wait) adds the partials in a fixed order, so the result does
// not depend on block scheduling.
#pragma once
#include <cuda_runtime.h>

namespace tog {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int NV, bool MAX = false>
__device__ __forceinline__ void block_reduce(double (&v)[NV], double (*sred)[32]) {
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nth = blockDim.x * blockDim.y * blockDim.z;
    const int lane = tid & 31, warp = tid >> 5, nw = (nth + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        v[i] = MAX ? warp_max(v[i]) : warp_sum(v[i]);
        if (lane == 0) sred[i][warp] = v[i];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double x = lane < nw ? sred[i][lane] : (MAX ? -1.0e308 : 0.0);
            x = MAX ? warp_max(x) : warp_sum(x);
            if (lane == 0) sred[i][0] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = sred[i][0];
    __syncthreads();
}

// Returns true in every thread of the last block; tot[] then holds the grid total.
template <int NV, bool MAX = false>
__device__ bool grid_reduce_last(double (&v)[NV], double* partials, unsigned* counter, double (&tot)[NV]) {
    __shared__ double sred[NV][32];
    __shared__ int amlast;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nth = blockDim.x * blockDim.y * blockDim.z;
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    block_reduce<NV, MAX>(v, sred);
    if (tid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[(size_t)bid * NV + i] = v[i];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        amlast = (t == nb - 1);
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) s[i] = MAX ? -1.0e308 : 0.0;
    for (unsigned b = tid; b < nb; b += nth) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double x = __ldcg(partials + (size_t)b * NV + i);
            s[i] = MAX ? fmax(s[i], x) : s[i] + x;
        }
    }
    block_reduce<NV, MAX>(s, sred);
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = s[i];
    if (tid == 0) *counter = 0u;
    return true;
}

}  // namespace tog
