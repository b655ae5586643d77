// Learned warm start: a small 3D convolutional encoder-decoder that maps the
// state of a SIMP design iteration on a structured hex8 grid (per node: the
// new filtered density, its change since the previous iteration, the previous
// displacement and its residual under the new densities, both scaled) to a
// correction of the previous displacement.  It has no counterpart in TopOpt.jl.
//
// Architecture (channels-last BF16 activations, every channel count padded to
// a multiple of 16, 3x3x3 kernels, zero padding 1):
//   e0: 16 -> 16, stride 1, ReLU          (level 0: the node grid)
//   e1: 16 -> 32, stride 2, ReLU          (level 1: (n + 1) / 2 per axis)
//   e2: 32 -> 48, stride 2, ReLU          (level 2)
//   e3: 48 -> 64, stride 2, ReLU          (level 3)
//   d2: up(e3) 64 -> 48, + e2, ReLU       (nearest x2 upsampling, skip added before the ReLU)
//   d1: up(d2) 48 -> 32, + e1, ReLU
//   d0: up(d1) 32 -> 16, + e0, ReLU
//   out: 16 -> 16 (3 used), no activation, FP32
// Input channels 0..7 (8..15 zero), output channels 0..2.
//
// Convolutions are implicit GEMMs on the tensor cores (mma.sync m16n8k16, BF16
// operands, FP32 accumulation): rows = output voxels, columns = output channels,
// reduction = 27 taps x input channels.  The same kernel computes the
// transposed convolution of the backward pass (input gradients); weight
// gradients are a split-K GEMM over voxels.  Training keeps FP32 master weights
// (Adam); the BF16 copies (and their transposes) are refreshed after each step.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "../../include/topopt_gb300.h"
#include "tog_internal.h"
#include "tog_nn.h"

using namespace tog;

namespace {

typedef __nv_bfloat16 bf16;

struct Vol {   // one activation volume: n samples x d x h x w voxels
    int n, d, h, w;
    __host__ __device__ long long vox() const { return (long long)n * d * h * w; }
};

struct ConvArgs {
    const void* A;       // gathered operand: input activation (forward) / output gradient (transposed)
    const bf16* B;       // weights [dst channel][27][src channel]
    void* out;           // dst tensor (dst vol x cdst)
    const float* bias;   // forward only (may be null)
    const bf16* skip;    // forward only: added before the activation (may be null)
    int relu;            // forward only
    int accumulate;      // FP32 output: out += result
    Vol src, dst;
    int csrc, cdst, stride;
};

struct WgradArgs {
    const float* dout;   // gradient of the forward output (out vol x cout), FP32
    const bf16* in;      // forward input (in vol x cin)
    float* dw;           // [cout][27][cin], accumulated
    Vol vin, vout;
    int cin, cout, stride;
    long long chunk;     // voxels per block
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t load_pair(const bf16* p, long long off, bool ok) {
    return ok ? *reinterpret_cast<const uint32_t*>(p + off) : 0u;
}
__device__ __forceinline__ uint32_t load_pair(const float* p, long long off, bool ok) {
    if (!ok) return 0u;
    const float2 v = *reinterpret_cast<const float2*>(p + off);
    return pack_bf16(v.x, v.y);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// voxel index -> (n, z, y, x)
__device__ __forceinline__ void vox_coords(const Vol& v, long long m, int& n, int& z, int& y, int& x) {
    x = (int)(m % v.w);
    long long r = m / v.w;
    y = (int)(r % v.h);
    r /= v.h;
    z = (int)(r % v.d);
    n = (int)(r / v.d);
}

// Source voxel of tap (kz, ky, kx) for destination voxel (n, z, y, x):
//   forward:    s = dst * stride + k - 1
//   transposed: dst = s * stride + k - 1 of the forward map, i.e. s = (dst + 1 - k) / stride
template <bool TRANSPOSED>
__device__ __forceinline__ bool src_voxel(const ConvArgs& a, int n, int z, int y, int x, int kz, int ky, int kx,
                                          long long& off) {
    int sz, sy, sx;
    if (!TRANSPOSED) {
        sz = z * a.stride + kz - 1;
        sy = y * a.stride + ky - 1;
        sx = x * a.stride + kx - 1;
    } else {
        const int tz = z + 1 - kz, ty = y + 1 - ky, tx = x + 1 - kx;
        if (tz < 0 || ty < 0 || tx < 0) return false;
        if (a.stride == 2 && ((tz | ty | tx) & 1)) return false;
        sz = tz / a.stride;
        sy = ty / a.stride;
        sx = tx / a.stride;
    }
    if (sz < 0 || sy < 0 || sx < 0 || sz >= a.src.d || sy >= a.src.h || sx >= a.src.w) return false;
    off = ((((long long)n * a.src.d + sz) * a.src.h + sy) * a.src.w + sx) * a.csrc;
    return true;
}

// Implicit-GEMM 3x3x3 convolution.  A warp computes 16 destination voxels x
// 8*NT destination channels (NT = cdst / 8), a block 4 warps.
template <typename TA, typename TO, int NT, bool TRANSPOSED>
__global__ void __launch_bounds__(128) k_conv(ConvArgs a) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const long long M = a.dst.vox();
    const long long m0 = ((long long)blockIdx.x * 4 + warp) * 16;
    if (m0 >= M) return;
    int rn[2], rz[2], ry[2], rx[2];
    bool rv[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const long long m = m0 + g + 8 * r;
        rv[r] = m < M;
        vox_coords(a.dst, rv[r] ? m : 0, rn[r], rz[r], ry[r], rx[r]);
    }
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const TA* A = reinterpret_cast<const TA*>(a.A);
    const int kchunks = a.csrc >> 4;
    const long long wstride = 27LL * a.csrc;   // one destination channel's weights
    for (int tap = 0; tap < 27; ++tap) {
        const int kz = tap / 9, ky = (tap / 3) % 3, kx = tap % 3;
        long long so[2] = {0, 0};
        bool sv[2];
#pragma unroll
        for (int r = 0; r < 2; ++r)
            sv[r] = rv[r] && src_voxel<TRANSPOSED>(a, rn[r], rz[r], ry[r], rx[r], kz, ky, kx, so[r]);
        if (!__any_sync(0xffffffffu, sv[0] || sv[1])) continue;
        for (int kc = 0; kc < kchunks; ++kc) {
            const int c0 = kc * 16 + 2 * t;
            const uint32_t a0 = load_pair(A, so[0] + c0, sv[0]);
            const uint32_t a1 = load_pair(A, so[1] + c0, sv[1]);
            const uint32_t a2 = load_pair(A, so[0] + c0 + 8, sv[0]);
            const uint32_t a3 = load_pair(A, so[1] + c0 + 8, sv[1]);
            const bf16* wb = a.B + (long long)tap * a.csrc + c0;
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const bf16* w = wb + (long long)(8 * j + g) * wstride;
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(w);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(w + 8);
                mma_bf16(acc[j], a0, a1, a2, a3, b0, b1);
            }
        }
    }
    // epilogue: rows m0 + g (c0, c1) and m0 + g + 8 (c2, c3), channels 8j + 2t, +1
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (!rv[r]) continue;
        const long long m = m0 + g + 8 * r;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int co = 8 * j + 2 * t;
            float v0 = acc[j][2 * r], v1 = acc[j][2 * r + 1];
            const long long o = m * a.cdst + co;
            if (a.bias) {
                v0 += a.bias[co];
                v1 += a.bias[co + 1];
            }
            if (a.skip) {
                const __nv_bfloat162 s = *reinterpret_cast<const __nv_bfloat162*>(a.skip + o);
                v0 += __low2float(s);
                v1 += __high2float(s);
            }
            if (a.relu) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            if constexpr (std::is_same<TO, float>::value) {
                float2* po = reinterpret_cast<float2*>(reinterpret_cast<float*>(a.out) + o);
                if (a.accumulate) {
                    const float2 old = *po;
                    v0 += old.x;
                    v1 += old.y;
                }
                *po = make_float2(v0, v1);
            } else {
                *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<bf16*>(a.out) + o) = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
}

// Weight gradient dW[co][tap][ci] += sum over forward-output voxels v of
// dout[v][co] * in[src(v, tap)][ci].  Block x = (tap, 16-channel block of co),
// block y = voxel chunk split over 4 warps; a warp covers 16 co x 8*NT ci
// (NT = cin / 8) and adds its partial sums with atomics.
template <int NT>
__global__ void __launch_bounds__(128) k_conv_wgrad(WgradArgs w) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int cot = blockIdx.x % (w.cout >> 4), tap = blockIdx.x / (w.cout >> 4);
    const int kz = tap / 9, ky = (tap / 3) % 3, kx = tap % 3;
    const int co0 = cot * 16;
    const long long M = w.vout.vox();
    const long long cb = (long long)blockIdx.y * w.chunk;
    const long long ce = (cb + w.chunk < M) ? cb + w.chunk : M;
    const long long per = (((ce - cb) + 63) / 64) * 16;   // 16-voxel steps per warp
    const long long vb = cb + warp * per, ve = (vb + per < ce) ? vb + per : ce;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    for (long long v0 = vb; v0 < ve; v0 += 16) {
        const long long va[4] = {v0 + 2 * t, v0 + 2 * t + 1, v0 + 2 * t + 8, v0 + 2 * t + 9};
        long long so[4];
        bool ok[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            ok[i] = va[i] < ve;
            so[i] = 0;
            if (ok[i]) {
                int n, z, y, x;
                vox_coords(w.vout, va[i], n, z, y, x);
                const int sz = z * w.stride + kz - 1, sy = y * w.stride + ky - 1, sx = x * w.stride + kx - 1;
                const bool in = sz >= 0 && sy >= 0 && sx >= 0 && sz < w.vin.d && sy < w.vin.h && sx < w.vin.w;
                so[i] = in ? ((((long long)n * w.vin.d + sz) * w.vin.h + sy) * w.vin.w + sx) * w.cin : -1;
            }
        }
        auto dv = [&](int i, int co) { return ok[i] ? w.dout[va[i] * w.cout + co] : 0.f; };
        const uint32_t a0 = pack_bf16(dv(0, co0 + g), dv(1, co0 + g));
        const uint32_t a1 = pack_bf16(dv(0, co0 + g + 8), dv(1, co0 + g + 8));
        const uint32_t a2 = pack_bf16(dv(2, co0 + g), dv(3, co0 + g));
        const uint32_t a3 = pack_bf16(dv(2, co0 + g + 8), dv(3, co0 + g + 8));
        auto iv = [&](int i, int ci) {
            return (ok[i] && so[i] >= 0) ? w.in[so[i] + ci] : __float2bfloat16(0.f);
        };
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int ci = 8 * j + g;
            __nv_bfloat162 p0, p1;
            p0.x = iv(0, ci);
            p0.y = iv(1, ci);
            p1.x = iv(2, ci);
            p1.y = iv(3, ci);
            mma_bf16(acc[j], a0, a1, a2, a3, *reinterpret_cast<uint32_t*>(&p0), *reinterpret_cast<uint32_t*>(&p1));
        }
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int ci = 8 * j + 2 * t;
        float* d0 = w.dw + ((long long)(co0 + g) * 27 + tap) * w.cin + ci;
        float* d1 = w.dw + ((long long)(co0 + g + 8) * 27 + tap) * w.cin + ci;
        atomicAdd(d0, acc[j][0]);
        atomicAdd(d0 + 1, acc[j][1]);
        atomicAdd(d1, acc[j][2]);
        atomicAdd(d1 + 1, acc[j][3]);
    }
}

// bias gradient: db[c] += sum_v g[v][c]
__global__ void k_bias_grad(const float* __restrict__ g, float* __restrict__ db, long long nvox, int c) {
    extern __shared__ float sb[];
    for (int i = threadIdx.x; i < c; i += blockDim.x) sb[i] = 0.f;
    __syncthreads();
    const long long n = nvox * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        atomicAdd(&sb[i % c], g[i]);
    __syncthreads();
    for (int i = threadIdx.x; i < c; i += blockDim.x) atomicAdd(&db[i], sb[i]);
}

// g *= (act > 0)
__global__ void k_relu_mask(float* __restrict__ g, const bf16* __restrict__ act, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(act[i]) > 0.f)) g[i] = 0.f;
}

// nearest x2 upsampling from coarse vol to fine vol (fine voxel z reads coarse z / 2)
__global__ void k_up(const bf16* __restrict__ src, bf16* __restrict__ dst, Vol vc, Vol vf, int c) {
    const long long n = vf.vox() * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        int s, z, y, x;
        vox_coords(vf, i / c, s, z, y, x);
        dst[i] = src[((((long long)s * vc.d + z / 2) * vc.h + y / 2) * vc.w + x / 2) * c + ch];
    }
}

// its adjoint: coarse gradient = sum of the fine gradients that read it
__global__ void k_up_bwd(const float* __restrict__ gf, float* __restrict__ gc, Vol vc, Vol vf, int c) {
    const long long n = vc.vox() * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        int s, z, y, x;
        vox_coords(vc, i / c, s, z, y, x);
        float acc = 0.f;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    const int fz = 2 * z + dz, fy = 2 * y + dy, fx = 2 * x + dx;
                    if (fz < vf.d && fy < vf.h && fx < vf.w)
                        acc += gf[((((long long)s * vf.d + fz) * vf.h + fy) * vf.w + fx) * c + ch];
                }
        gc[i] = acc;
    }
}

// network input: FP32 (vox x 8) -> BF16 (vox x 16), channels 8..15 zero
__global__ void k_pack_input(const float* __restrict__ in, bf16* __restrict__ x, long long nvox) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[v * 16 + c] = __float2bfloat16(in[v * 8 + c]);
#pragma unroll
        for (int c = 8; c < 16; ++c) x[v * 16 + c] = __float2bfloat16(0.f);
    }
}

__global__ void k_unpack_output(const float* __restrict__ y, float* __restrict__ out, long long nvox) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
        out[v * 3] = y[v * 16];
        out[v * 3 + 1] = y[v * 16 + 1];
        out[v * 3 + 2] = y[v * 16 + 2];
    }
}

// mean squared error over vox x 3 and its gradient into dy (vox x 16)
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ tgt, float* __restrict__ dy, long long nvox,
                      double* __restrict__ loss) {
    const double inv = 1.0 / (3.0 * (double)nvox);
    double s = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            float gval = 0.f;
            if (c < 3) {
                const float e = y[v * 16 + c] - tgt[v * 3 + c];
                s += (double)e * e;
                gval = (float)(2.0 * inv) * e;
            }
            dy[v * 16 + c] = gval;
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv);
}

// BF16 weight copies: B [co][27][ci] and its transpose [ci][27][co]
__global__ void k_weights_bf16(const float* __restrict__ w, bf16* __restrict__ b, bf16* __restrict__ bt, int cout,
                               int cin) {
    const long long n = 27LL * cout * cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const int tap = (int)((i / cin) % 27);
        const int co = (int)(i / (27LL * cin));
        const bf16 v = __float2bfloat16(w[i]);
        b[i] = v;
        bt[((long long)ci * 27 + tap) * cout + co] = v;
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

struct ConvLayer {
    int cin, cout, stride;
    long long woff, boff;   // offsets of W and b in the parameter vector
};

int nn_fail(int code, const std::string& m) { return tog::set_error(code, m.c_str()); }

#define NN_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return nn_fail(e_ == cudaErrorMemoryAllocation ? TOG_ERR_OOM : TOG_ERR_CUDA,                 \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

}  // namespace

struct tog_nn {
    Vol lv[4];                      // level volumes (batch included)
    int nodes[3];
    ConvLayer L[8];
    long long nparam = 0;
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    bf16 *d_wb = nullptr, *d_wt = nullptr;   // bf16 copies of all W (same offsets as the fp32 vector)
    // activations (bf16)
    bf16 *x0 = nullptr, *a0 = nullptr, *a1 = nullptr, *a2 = nullptr, *a3 = nullptr;
    bf16 *u2 = nullptr, *b2 = nullptr, *u1 = nullptr, *b1 = nullptr, *u0 = nullptr, *b0 = nullptr;
    float* y = nullptr;             // output (vox0 x 16)
    // gradients (fp32)
    float *gy = nullptr, *g0 = nullptr, *g0b = nullptr, *gu0 = nullptr, *g1 = nullptr, *g1b = nullptr, *gu1 = nullptr;
    float *g2 = nullptr, *g2b = nullptr, *gu2 = nullptr, *g3 = nullptr;
    double* d_loss = nullptr;
    std::vector<void*> allocs;
    cudaStream_t stream = nullptr;
    int steps = 0;
    int nsm = 152;
};

namespace {

template <typename T>
int nalloc(tog_nn* nn, T** p, long long n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<long long>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return nn_fail(TOG_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    nn->allocs.push_back(*p);
    return TOG_OK;
}

int ew_grid(const tog_nn* nn, long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)nn->nsm * 16));
}

template <typename TA, typename TO, bool TR>
void conv_launch(const ConvArgs& a, cudaStream_t s) {
    const long long M = a.dst.vox();
    const int grid = (int)((M + 63) / 64);
    switch (a.cdst / 8) {
        case 2: k_conv<TA, TO, 2, TR><<<grid, 128, 0, s>>>(a); break;
        case 4: k_conv<TA, TO, 4, TR><<<grid, 128, 0, s>>>(a); break;
        case 6: k_conv<TA, TO, 6, TR><<<grid, 128, 0, s>>>(a); break;
        default: k_conv<TA, TO, 8, TR><<<grid, 128, 0, s>>>(a); break;
    }
}

// forward convolution of layer l from `in` (vol vi) to `out` (vol vo)
template <typename TO>
void conv_fwd(tog_nn* nn, int l, const bf16* in, Vol vi, void* out, Vol vo, const bf16* skip, int relu) {
    const ConvLayer& C = nn->L[l];
    ConvArgs a{};
    a.A = in;
    a.B = nn->d_wb + C.woff;
    a.out = out;
    a.bias = nn->d_p + C.boff;
    a.skip = skip;
    a.relu = relu;
    a.src = vi;
    a.dst = vo;
    a.csrc = C.cin;
    a.cdst = C.cout;
    a.stride = C.stride;
    conv_launch<bf16, TO, false>(a, nn->stream);
}

// input gradient of layer l: gin (vol vi, cin) (+)= conv^T(gout (vol vo, cout))
void conv_bwd_data(tog_nn* nn, int l, const float* gout, Vol vo, float* gin, Vol vi, int accumulate) {
    const ConvLayer& C = nn->L[l];
    ConvArgs a{};
    a.A = gout;
    a.B = nn->d_wt + C.woff;
    a.out = gin;
    a.accumulate = accumulate;
    a.src = vo;
    a.dst = vi;
    a.csrc = C.cout;
    a.cdst = C.cin;
    a.stride = C.stride;
    conv_launch<float, float, true>(a, nn->stream);
}

void conv_wgrad(tog_nn* nn, int l, const float* gout, Vol vo, const bf16* in, Vol vi) {
    const ConvLayer& C = nn->L[l];
    WgradArgs w{};
    w.dout = gout;
    w.in = in;
    w.dw = nn->d_g + C.woff;
    w.vin = vi;
    w.vout = vo;
    w.cin = C.cin;
    w.cout = C.cout;
    w.stride = C.stride;
    const long long M = vo.vox();
    const long long want = std::max<long long>(1, (long long)nn->nsm * 8 / (27 * (C.cout / 16)));
    w.chunk = std::max<long long>(64, ((M + want - 1) / want + 63) / 64 * 64);
    dim3 grid(27 * (C.cout / 16), (unsigned)((M + w.chunk - 1) / w.chunk));
    switch (C.cin / 8) {
        case 2: k_conv_wgrad<2><<<grid, 128, 0, nn->stream>>>(w); break;
        case 4: k_conv_wgrad<4><<<grid, 128, 0, nn->stream>>>(w); break;
        case 6: k_conv_wgrad<6><<<grid, 128, 0, nn->stream>>>(w); break;
        default: k_conv_wgrad<8><<<grid, 128, 0, nn->stream>>>(w); break;
    }
    k_bias_grad<<<ew_grid(nn, M * C.cout), 256, C.cout * sizeof(float), nn->stream>>>(gout, nn->d_g + C.boff, M,
                                                                                      C.cout);
}

void forward(tog_nn* nn, const float* in) {
    cudaStream_t s = nn->stream;
    const Vol* V = nn->lv;
    k_pack_input<<<ew_grid(nn, V[0].vox()), 256, 0, s>>>(in, nn->x0, V[0].vox());
    conv_fwd<bf16>(nn, 0, nn->x0, V[0], nn->a0, V[0], nullptr, 1);
    conv_fwd<bf16>(nn, 1, nn->a0, V[0], nn->a1, V[1], nullptr, 1);
    conv_fwd<bf16>(nn, 2, nn->a1, V[1], nn->a2, V[2], nullptr, 1);
    conv_fwd<bf16>(nn, 3, nn->a2, V[2], nn->a3, V[3], nullptr, 1);
    k_up<<<ew_grid(nn, V[2].vox() * 64), 256, 0, s>>>(nn->a3, nn->u2, V[3], V[2], 64);
    conv_fwd<bf16>(nn, 4, nn->u2, V[2], nn->b2, V[2], nn->a2, 1);
    k_up<<<ew_grid(nn, V[1].vox() * 48), 256, 0, s>>>(nn->b2, nn->u1, V[2], V[1], 48);
    conv_fwd<bf16>(nn, 5, nn->u1, V[1], nn->b1, V[1], nn->a1, 1);
    k_up<<<ew_grid(nn, V[0].vox() * 32), 256, 0, s>>>(nn->b1, nn->u0, V[1], V[0], 32);
    conv_fwd<bf16>(nn, 6, nn->u0, V[0], nn->b0, V[0], nn->a0, 1);
    conv_fwd<float>(nn, 7, nn->b0, V[0], nn->y, V[0], nullptr, 0);
}

// gradients of the mean squared error w.r.t. all parameters (into d_g)
int backward(tog_nn* nn, const float* tgt, double* loss_host) {
    cudaStream_t s = nn->stream;
    const Vol* V = nn->lv;
    NN_CUDA(cudaMemsetAsync(nn->d_g, 0, nn->nparam * sizeof(float), s));
    NN_CUDA(cudaMemsetAsync(nn->d_loss, 0, sizeof(double), s));
    const long long n0 = V[0].vox(), n1 = V[1].vox(), n2 = V[2].vox(), n3 = V[3].vox();
    k_mse<<<ew_grid(nn, n0), 256, 0, s>>>(nn->y, tgt, nn->gy, n0, nn->d_loss);
    // out
    conv_wgrad(nn, 7, nn->gy, V[0], nn->b0, V[0]);
    conv_bwd_data(nn, 7, nn->gy, V[0], nn->g0b, V[0], 0);
    k_relu_mask<<<ew_grid(nn, n0 * 16), 256, 0, s>>>(nn->g0b, nn->b0, n0 * 16);   // dz at d0 (also the a0 skip)
    // d0
    conv_wgrad(nn, 6, nn->g0b, V[0], nn->u0, V[0]);
    conv_bwd_data(nn, 6, nn->g0b, V[0], nn->gu0, V[0], 0);
    k_up_bwd<<<ew_grid(nn, n1 * 32), 256, 0, s>>>(nn->gu0, nn->g1b, V[1], V[0], 32);
    k_relu_mask<<<ew_grid(nn, n1 * 32), 256, 0, s>>>(nn->g1b, nn->b1, n1 * 32);
    // d1
    conv_wgrad(nn, 5, nn->g1b, V[1], nn->u1, V[1]);
    conv_bwd_data(nn, 5, nn->g1b, V[1], nn->gu1, V[1], 0);
    k_up_bwd<<<ew_grid(nn, n2 * 48), 256, 0, s>>>(nn->gu1, nn->g2b, V[2], V[1], 48);
    k_relu_mask<<<ew_grid(nn, n2 * 48), 256, 0, s>>>(nn->g2b, nn->b2, n2 * 48);
    // d2
    conv_wgrad(nn, 4, nn->g2b, V[2], nn->u2, V[2]);
    conv_bwd_data(nn, 4, nn->g2b, V[2], nn->gu2, V[2], 0);
    k_up_bwd<<<ew_grid(nn, n3 * 64), 256, 0, s>>>(nn->gu2, nn->g3, V[3], V[2], 64);
    k_relu_mask<<<ew_grid(nn, n3 * 64), 256, 0, s>>>(nn->g3, nn->a3, n3 * 64);
    // e3: the gradient of a2 = skip part (g2b) + conv^T part
    conv_wgrad(nn, 3, nn->g3, V[3], nn->a2, V[2]);
    NN_CUDA(cudaMemcpyAsync(nn->g2, nn->g2b, n2 * 48 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    conv_bwd_data(nn, 3, nn->g3, V[3], nn->g2, V[2], 1);
    k_relu_mask<<<ew_grid(nn, n2 * 48), 256, 0, s>>>(nn->g2, nn->a2, n2 * 48);
    // e2
    conv_wgrad(nn, 2, nn->g2, V[2], nn->a1, V[1]);
    NN_CUDA(cudaMemcpyAsync(nn->g1, nn->g1b, n1 * 32 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    conv_bwd_data(nn, 2, nn->g2, V[2], nn->g1, V[1], 1);
    k_relu_mask<<<ew_grid(nn, n1 * 32), 256, 0, s>>>(nn->g1, nn->a1, n1 * 32);
    // e1
    conv_wgrad(nn, 1, nn->g1, V[1], nn->a0, V[0]);
    NN_CUDA(cudaMemcpyAsync(nn->g0, nn->g0b, n0 * 16 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    conv_bwd_data(nn, 1, nn->g1, V[1], nn->g0, V[0], 1);
    k_relu_mask<<<ew_grid(nn, n0 * 16), 256, 0, s>>>(nn->g0, nn->a0, n0 * 16);
    // e0
    conv_wgrad(nn, 0, nn->g0, V[0], nn->x0, V[0]);
    NN_CUDA(cudaGetLastError());
    if (loss_host) {
        NN_CUDA(cudaMemcpyAsync(loss_host, nn->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
        NN_CUDA(cudaStreamSynchronize(s));
    }
    return TOG_OK;
}

void refresh_bf16(tog_nn* nn) {
    for (int l = 0; l < 8; ++l) {
        const ConvLayer& C = nn->L[l];
        k_weights_bf16<<<ew_grid(nn, 27LL * C.cin * C.cout), 256, 0, nn->stream>>>(
            nn->d_p + C.woff, nn->d_wb + C.woff, nn->d_wt + C.woff, C.cout, C.cin);
    }
}

}  // namespace

namespace tog {

int nn_forward_dev(tog_nn* nn, const float* in_dev, float* out_dev, cudaStream_t stream) {
    cudaStream_t keep = nn->stream;
    nn->stream = stream;
    forward(nn, in_dev);
    k_unpack_output<<<ew_grid(nn, nn->lv[0].vox()), 256, 0, stream>>>(nn->y, out_dev, nn->lv[0].vox());
    nn->stream = keep;
    NN_CUDA(cudaGetLastError());
    return TOG_OK;
}

bool nn_matches(const tog_nn* nn, const int nodes[3], int batch) {
    return nn && nn->nodes[0] == nodes[0] && nn->nodes[1] == nodes[1] && nn->nodes[2] == nodes[2] &&
           nn->lv[0].n == batch;
}

}  // namespace tog

extern "C" {

int tog_nn_create(const int32_t nodes[3], int32_t batch, uint64_t seed, tog_nn** out) {
    if (!out || !nodes || batch < 1 || nodes[0] < 2 || nodes[1] < 2 || nodes[2] < 2)
        return nn_fail(TOG_ERR_ARG, "tog_nn_create: bad arguments");
    *out = nullptr;
    tog_nn* nn = new tog_nn();
    for (int i = 0; i < 3; ++i) nn->nodes[i] = nodes[i];
    nn->lv[0] = Vol{batch, nodes[2], nodes[1], nodes[0]};
    for (int l = 1; l < 4; ++l)
        nn->lv[l] = Vol{batch, (nn->lv[l - 1].d + 1) / 2, (nn->lv[l - 1].h + 1) / 2, (nn->lv[l - 1].w + 1) / 2};
    const int spec[8][3] = {{16, 16, 1}, {16, 32, 2}, {32, 48, 2}, {48, 64, 2},
                            {64, 48, 1}, {48, 32, 1}, {32, 16, 1}, {16, 16, 1}};
    long long off = 0;
    for (int l = 0; l < 8; ++l) {
        nn->L[l] = ConvLayer{spec[l][0], spec[l][1], spec[l][2], off, off + 27LL * spec[l][0] * spec[l][1]};
        off = nn->L[l].boff + spec[l][1];
    }
    nn->nparam = off;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nn->nsm, cudaDevAttrMultiProcessorCount, dev);
    int rc = TOG_OK;
    auto R = [&](int r) {
        if (rc == TOG_OK) rc = r;
    };
    const long long n0 = nn->lv[0].vox(), n1 = nn->lv[1].vox(), n2 = nn->lv[2].vox(), n3 = nn->lv[3].vox();
    R(nalloc(nn, &nn->d_p, off));
    R(nalloc(nn, &nn->d_g, off));
    R(nalloc(nn, &nn->d_m, off));
    R(nalloc(nn, &nn->d_v, off));
    R(nalloc(nn, &nn->d_wb, off));
    R(nalloc(nn, &nn->d_wt, off));
    R(nalloc(nn, &nn->x0, n0 * 16));
    R(nalloc(nn, &nn->a0, n0 * 16));
    R(nalloc(nn, &nn->a1, n1 * 32));
    R(nalloc(nn, &nn->a2, n2 * 48));
    R(nalloc(nn, &nn->a3, n3 * 64));
    R(nalloc(nn, &nn->u2, n2 * 64));
    R(nalloc(nn, &nn->b2, n2 * 48));
    R(nalloc(nn, &nn->u1, n1 * 48));
    R(nalloc(nn, &nn->b1, n1 * 32));
    R(nalloc(nn, &nn->u0, n0 * 32));
    R(nalloc(nn, &nn->b0, n0 * 16));
    R(nalloc(nn, &nn->y, n0 * 16));
    R(nalloc(nn, &nn->gy, n0 * 16));
    R(nalloc(nn, &nn->g0, n0 * 16));
    R(nalloc(nn, &nn->g0b, n0 * 16));
    R(nalloc(nn, &nn->gu0, n0 * 32));
    R(nalloc(nn, &nn->g1, n1 * 32));
    R(nalloc(nn, &nn->g1b, n1 * 32));
    R(nalloc(nn, &nn->gu1, n1 * 48));
    R(nalloc(nn, &nn->g2, n2 * 48));
    R(nalloc(nn, &nn->g2b, n2 * 48));
    R(nalloc(nn, &nn->gu2, n2 * 64));
    R(nalloc(nn, &nn->g3, n3 * 64));
    R(nalloc(nn, &nn->d_loss, 1));
    if (rc != TOG_OK) {
        std::string m = tog_last_error();
        tog_nn_destroy(nn);
        nn_fail(rc, m);
        return rc;
    }
    // He-normal weights (the last layer's unused output channels zero), zero biases
    std::vector<float> h(off, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < 8; ++l) {
        const ConvLayer& C = nn->L[l];
        const int fan_in = 27 * (l == 0 ? 8 : C.cin);
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / fan_in) * (l == 7 ? 0.1f : 1.f));
        for (int co = 0; co < C.cout; ++co)
            for (int tap = 0; tap < 27; ++tap)
                for (int ci = 0; ci < C.cin; ++ci) {
                    const bool used = !(l == 0 && ci >= 8) && !(l == 7 && co >= 3);
                    h[C.woff + ((long long)co * 27 + tap) * C.cin + ci] = used ? nd(rng) : 0.f;
                }
    }
    cudaError_t e = cudaMemcpy(nn->d_p, h.data(), off * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(nn->d_m, 0, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(nn->d_v, 0, off * sizeof(float));
    if (e == cudaSuccess) {
        refresh_bf16(nn);
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        tog_nn_destroy(nn);
        return nn_fail(TOG_ERR_CUDA, std::string("tog_nn_create: ") + cudaGetErrorString(e));
    }
    *out = nn;
    return TOG_OK;
}

int tog_nn_destroy(tog_nn* nn) {
    if (!nn) return TOG_OK;
    if (nn->stream) cudaStreamSynchronize(nn->stream);
    for (void* p : nn->allocs) cudaFree(p);
    delete nn;
    return TOG_OK;
}

int tog_nn_set_stream(tog_nn* nn, void* stream) {
    if (!nn) return nn_fail(TOG_ERR_ARG, "null network");
    nn->stream = (cudaStream_t)stream;
    return TOG_OK;
}

int tog_nn_param_count(const tog_nn* nn, int64_t* count) {
    if (!nn || !count) return nn_fail(TOG_ERR_ARG, "null argument");
    *count = nn->nparam;
    return TOG_OK;
}

int tog_nn_get_params(tog_nn* nn, float* params) {
    if (!nn || !params) return nn_fail(TOG_ERR_ARG, "null argument");
    NN_CUDA(cudaMemcpyAsync(params, nn->d_p, nn->nparam * sizeof(float), cudaMemcpyDeviceToHost, nn->stream));
    NN_CUDA(cudaStreamSynchronize(nn->stream));
    return TOG_OK;
}

int tog_nn_set_params(tog_nn* nn, const float* params) {
    if (!nn || !params) return nn_fail(TOG_ERR_ARG, "null argument");
    NN_CUDA(cudaMemcpyAsync(nn->d_p, params, nn->nparam * sizeof(float), cudaMemcpyHostToDevice, nn->stream));
    NN_CUDA(cudaMemsetAsync(nn->d_m, 0, nn->nparam * sizeof(float), nn->stream));
    NN_CUDA(cudaMemsetAsync(nn->d_v, 0, nn->nparam * sizeof(float), nn->stream));
    nn->steps = 0;
    refresh_bf16(nn);
    NN_CUDA(cudaStreamSynchronize(nn->stream));
    return TOG_OK;
}

int tog_nn_forward(tog_nn* nn, const float* in_dev, float* out_dev) {
    if (!nn || !in_dev || !out_dev) return nn_fail(TOG_ERR_ARG, "null argument");
    return nn_forward_dev(nn, in_dev, out_dev, nn->stream);
}

int tog_nn_gradients(tog_nn* nn, const float* in_dev, const float* target_dev, double* loss, float* grads) {
    if (!nn || !in_dev || !target_dev) return nn_fail(TOG_ERR_ARG, "null argument");
    forward(nn, in_dev);
    double l = 0.0;
    int rc = backward(nn, target_dev, &l);
    if (rc != TOG_OK) return rc;
    if (loss) *loss = l;
    if (grads) {
        NN_CUDA(cudaMemcpyAsync(grads, nn->d_g, nn->nparam * sizeof(float), cudaMemcpyDeviceToHost, nn->stream));
        NN_CUDA(cudaStreamSynchronize(nn->stream));
    }
    return TOG_OK;
}

int tog_nn_train_step(tog_nn* nn, const float* in_dev, const float* target_dev, float lr, double* loss) {
    if (!nn || !in_dev || !target_dev || !(lr > 0.f)) return nn_fail(TOG_ERR_ARG, "bad argument");
    forward(nn, in_dev);
    int rc = backward(nn, target_dev, loss);
    if (rc != TOG_OK) return rc;
    nn->steps += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f / (1.f - std::pow(b1, (float)nn->steps)), c2 = 1.f / (1.f - std::pow(b2, (float)nn->steps));
    k_adam<<<ew_grid(nn, nn->nparam), 256, 0, nn->stream>>>(nn->d_p, nn->d_g, nn->d_m, nn->d_v, nn->nparam, lr, b1, b2,
                                                            1e-8f, c1, c2);
    refresh_bf16(nn);
    NN_CUDA(cudaGetLastError());
    return TOG_OK;
}

}  // extern "C"
