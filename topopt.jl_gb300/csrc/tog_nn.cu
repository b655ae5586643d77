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
// Convolutions are implicit GEMMs on the tcgen05 tensor cores (kind::f16, BF16
// operands staged in shared memory, FP32 accumulators in TMEM; tog_tc.cuh): rows =
// output voxels, columns = output channels, reduction = 27 taps x input channels.
// The same kernel computes the transposed convolution of the backward pass (input
// gradients); weight gradients are a GEMM with rows = (tap, input channel), columns =
// output channels and the reduction over voxels, split over blocks.  Training keeps
// FP32 master weights (Adam); the BF16 copies (and their transposes) are refreshed
// after each step.
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
#include "tog_tc.cuh"

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

// Eight consecutive channels of the gathered operand as BF16 (16 bytes).
__device__ __forceinline__ uint4 load8(const bf16* p, long long off) {
    return *reinterpret_cast<const uint4*>(p + off);
}
__device__ __forceinline__ uint4 load8(const float* p, long long off) {
    const float4 a = *reinterpret_cast<const float4*>(p + off);
    const float4 b = *reinterpret_cast<const float4*>(p + off + 4);
    return make_uint4(pack_bf16(a.x, a.y), pack_bf16(a.z, a.w), pack_bf16(b.x, b.y), pack_bf16(b.z, b.w));
}

constexpr int kTcRows = 128;        // destination voxels of a block (the MMA's M)

// Shared memory of k_conv_tc: two stages of (A: 128 x csrc, B: cdst x csrc) BF16, two mbarriers
// and the TMEM address slot.
inline size_t conv_tc_smem(int csrc, int cdst) {
    return 2 * ((size_t)kTcRows * csrc * 2 + (size_t)cdst * csrc * 2) + 32;
}

// Implicit-GEMM 3x3x3 convolution on the tcgen05 tensor cores.  A block owns 128
// destination voxels (one per thread) and all N = cdst destination channels; the FP32
// accumulator (128 x N) lives in TMEM.  Per tap each thread gathers its voxel's source
// channels (BF16, zero outside the volume) into the A stage in shared memory, the block
// copies the tap's weights into the B stage, and one thread issues csrc / 16 MMAs and
// commits them to the stage's mbarrier; the two stages alternate, so the gather of a
// tap overlaps the MMAs of the previous one.  The epilogue reads each thread's row
// back from TMEM (bias, skip, ReLU, store).  Every wait is bounded: on a timeout the
// block stops issuing, waits (bounded) for what it issued, frees its TMEM, sets *err
// and returns.
template <typename TA, typename TO, int N, bool TRANSPOSED>
__global__ void __launch_bounds__(kTcRows) k_conv_tc(ConvArgs a, int* err) {
    extern __shared__ __align__(128) uint8_t tsm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int K = a.csrc;
    const uint32_t abytes = (uint32_t)kTcRows * K * 2, bbytes = (uint32_t)N * K * 2, sbo = (uint32_t)K * 16;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + 2 * (abytes + bbytes));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    constexpr uint32_t kCols = N <= 32 ? 32 : 64;
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(tslot, kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;

    const long long M = a.dst.vox();
    const long long m = (long long)blockIdx.x * kTcRows + tid;
    const bool rv = m < M;
    int rn, rz, ry, rx;
    vox_coords(a.dst, rv ? m : 0, rn, rz, ry, rx);
    const TA* A = reinterpret_cast<const TA*>(a.A);
    const int kc8 = K >> 3;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kTcRows, N);
    int issued0 = 0, issued1 = 0;   // commits per stage
    bool fail = false;
    for (int tap = 0; tap < 27; ++tap) {
        const int s = tap & 1;
        const int iss = s ? issued1 : issued0;
        if (iss > 0) fail = !tc::mbar_wait(&bar[s], (iss - 1) & 1, tc::kTcWaitPolls);
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        const int kz = tap / 9, ky = (tap / 3) % 3, kx = tap % 3;
        long long so = 0;
        const bool sv = rv && src_voxel<TRANSPOSED>(a, rn, rz, ry, rx, kz, ky, kx, so);
        uint8_t* const sa_p = tsm + s * (abytes + bbytes);
        uint8_t* arow = sa_p + (tid >> 3) * sbo + (tid & 7) * 16;
        for (int kc = 0; kc < kc8; ++kc)
            *reinterpret_cast<uint4*>(arow + kc * 128) = sv ? load8(A, so + 8 * kc) : make_uint4(0, 0, 0, 0);
        uint8_t* bt = sa_p + abytes;
        for (int i = tid; i < N * kc8; i += kTcRows) {
            const int n = i / kc8, kc = i - n * kc8;
            *reinterpret_cast<uint4*>(bt + (n >> 3) * sbo + kc * 128 + (n & 7) * 16) =
                *reinterpret_cast<const uint4*>(a.B + ((long long)n * 27 + tap) * K + 8 * kc);
        }
        tc::fence_async_shared();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t sa = tc::smem_u32(sa_p), sb = tc::smem_u32(bt);
            for (int kc = 0; kc < (K >> 4); ++kc)
                tc::mma_bf16(tmem, tc::smem_desc(sa + kc * 256, 128, sbo), tc::smem_desc(sb + kc * 256, 128, sbo),
                             idesc, (tap | kc) != 0);
            tc::mma_commit(&bar[s]);
        }
        if (s) ++issued1; else ++issued0;
    }
    // every issued MMA has completed once the last commit of each stage has
    bool drained = true;
    if (issued0 > 0) drained = tc::mbar_wait(&bar[0], (issued0 - 1) & 1, tc::kTcWaitPolls) && drained;
    if (issued1 > 0) drained = tc::mbar_wait(&bar[1], (issued1 - 1) & 1, tc::kTcWaitPolls) && drained;
    drained = __syncthreads_and(drained);
    tc::fence_after_sync();
    if (!fail && drained) {   // block-uniform: the TMEM loads are warp-collective
        float acc[N];
#pragma unroll
        for (int c = 0; c < N; c += 16) tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c, acc + c);
        const long long o = m * a.cdst;
#pragma unroll
        for (int c = 0; c < N; c += 8) {
            if (!rv) break;
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = acc[c + i] + (a.bias ? a.bias[c + i] : 0.f);
            if (a.skip) {
                const uint4 sk = *reinterpret_cast<const uint4*>(a.skip + o + c);
                const __nv_bfloat162* s2 = reinterpret_cast<const __nv_bfloat162*>(&sk);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    v[2 * i] += __low2float(s2[i]);
                    v[2 * i + 1] += __high2float(s2[i]);
                }
            }
            if (a.relu) {
#pragma unroll
                for (int i = 0; i < 8; ++i) v[i] = fmaxf(v[i], 0.f);
            }
            if constexpr (std::is_same<TO, float>::value) {
                float4* po = reinterpret_cast<float4*>(reinterpret_cast<float*>(a.out) + o + c);
                if (a.accumulate) {
                    const float4 p0 = po[0], p1 = po[1];
                    v[0] += p0.x, v[1] += p0.y, v[2] += p0.z, v[3] += p0.w;
                    v[4] += p1.x, v[5] += p1.y, v[6] += p1.z, v[7] += p1.w;
                }
                po[0] = make_float4(v[0], v[1], v[2], v[3]);
                po[1] = make_float4(v[4], v[5], v[6], v[7]);
            } else {
                *reinterpret_cast<uint4*>(reinterpret_cast<bf16*>(a.out) + o + c) =
                    make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kCols);
    }
    if (tid == 0 && (fail || !drained)) atomicExch(err, 1);
}

constexpr int kWgVox = 64;   // voxels per stage of k_wgrad_tc (four K = 16 MMAs)

inline size_t wgrad_tc_smem(int cout) { return 2 * ((size_t)kTcRows * kWgVox * 2 + (size_t)cout * kWgVox * 2) + 32; }

// Weight gradient on the tcgen05 tensor cores: dW[co][tap][ci] += sum over forward-output
// voxels v of dout[v][co] * in[src(v, tap)][ci].  MMA rows are 128 consecutive (tap, ci)
// pairs of the 27 * cin (block x), columns the N = cout output channels, the reduction runs
// over the block's voxel range (block y) 64 voxels per stage.  Both operands are written
// K-major (voxels contiguous inside a core matrix) by the threads: a thread owns one voxel
// of the stage and scatters its 8-channel groups down the rows.  The FP32 accumulator
// stays in TMEM until the end, then every thread adds its row to dW with atomics.  Waits
// are bounded as in k_conv_tc.
template <int N>
__global__ void __launch_bounds__(kTcRows) k_wgrad_tc(WgradArgs w, int* err) {
    extern __shared__ __align__(128) uint8_t tsm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t abytes = kTcRows * kWgVox * 2, bbytes = N * kWgVox * 2, sbo = kWgVox * 16;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + 2 * (abytes + bbytes));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    constexpr uint32_t kCols = N <= 32 ? 32 : 64;
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(tslot, kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;

    const int rows = 27 * w.cin;
    const int r0 = blockIdx.x * kTcRows;   // first (tap, ci) row of the block
    const long long M = w.vout.vox();
    const long long cb = (long long)blockIdx.y * w.chunk;
    const long long ce = cb + w.chunk < M ? cb + w.chunk : M;
    const int nst = (int)((ce - cb + kWgVox - 1) / kWgVox);
    const int vl = tid & (kWgVox - 1), gh = tid / kWgVox;   // voxel of the stage, half of the row groups
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kTcRows, N);
    int issued0 = 0, issued1 = 0;
    bool fail = false;
    for (int it = 0; it < nst; ++it) {
        const int s = it & 1;
        const int iss = s ? issued1 : issued0;
        if (iss > 0) fail = !tc::mbar_wait(&bar[s], (iss - 1) & 1, tc::kTcWaitPolls);
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        uint8_t* const sa_p = tsm + s * (abytes + bbytes);
        uint8_t* const sb_p = sa_p + abytes;
        const long long v = cb + (long long)it * kWgVox + vl;
        const bool vok = v < ce;
        int n = 0, z = 0, y = 0, x = 0;
        if (vok) vox_coords(w.vout, v, n, z, y, x);
        const uint32_t col = (vl >> 3) * 128 + (vl & 7) * 2;   // this voxel's column in a core matrix row group
        // A: 16 groups of 8 rows (tap, ci..ci+7); this thread fills 8 of them for its voxel
#pragma unroll 2
        for (int g = gh; g < kTcRows / 8; g += kTcRows / kWgVox) {
            const int r = r0 + 8 * g;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (vok && r < rows) {
                const int tap = r / w.cin, ci = r - tap * w.cin;
                const int kz = tap / 9, ky = (tap / 3) % 3, kx = tap % 3;
                const int sz = z * w.stride + kz - 1, sy = y * w.stride + ky - 1, sx = x * w.stride + kx - 1;
                if (sz >= 0 && sy >= 0 && sx >= 0 && sz < w.vin.d && sy < w.vin.h && sx < w.vin.w)
                    val = *reinterpret_cast<const uint4*>(
                        w.in + ((((long long)n * w.vin.d + sz) * w.vin.h + sy) * w.vin.w + sx) * w.cin + ci);
            }
            const uint16_t* h = reinterpret_cast<const uint16_t*>(&val);
            uint8_t* dst = sa_p + g * sbo + col;
#pragma unroll
            for (int i = 0; i < 8; ++i) *reinterpret_cast<uint16_t*>(dst + i * 16) = h[i];
        }
        // B: N / 8 groups of 8 output channels of dout (FP32 -> BF16)
        for (int g = gh; g < N / 8; g += kTcRows / kWgVox) {
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
            if (vok) {
                const float4* src = reinterpret_cast<const float4*>(w.dout + v * w.cout + 8 * g);
                a = src[0];
                b = src[1];
            }
            const bf16 hv[8] = {__float2bfloat16(a.x), __float2bfloat16(a.y), __float2bfloat16(a.z),
                                __float2bfloat16(a.w), __float2bfloat16(b.x), __float2bfloat16(b.y),
                                __float2bfloat16(b.z), __float2bfloat16(b.w)};
            uint8_t* dst = sb_p + g * sbo + col;
#pragma unroll
            for (int i = 0; i < 8; ++i) *reinterpret_cast<bf16*>(dst + i * 16) = hv[i];
        }
        tc::fence_async_shared();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t sa = tc::smem_u32(sa_p), sb = tc::smem_u32(sb_p);
#pragma unroll
            for (int kc = 0; kc < kWgVox / 16; ++kc)
                tc::mma_bf16(tmem, tc::smem_desc(sa + kc * 256, 128, sbo), tc::smem_desc(sb + kc * 256, 128, sbo),
                             idesc, (it | kc) != 0);
            tc::mma_commit(&bar[s]);
        }
        if (s) ++issued1; else ++issued0;
    }
    bool drained = true;
    if (issued0 > 0) drained = tc::mbar_wait(&bar[0], (issued0 - 1) & 1, tc::kTcWaitPolls) && drained;
    if (issued1 > 0) drained = tc::mbar_wait(&bar[1], (issued1 - 1) & 1, tc::kTcWaitPolls) && drained;
    drained = __syncthreads_and(drained);
    tc::fence_after_sync();
    if (!fail && drained && nst > 0) {   // block-uniform: the TMEM loads are warp-collective
        float acc[N];
#pragma unroll
        for (int c = 0; c < N; c += 16) tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c, acc + c);
        const int r = r0 + tid;
        if (r < rows) {
            const int tap = r / w.cin, ci = r - tap * w.cin;
#pragma unroll
            for (int co = 0; co < N; ++co) atomicAdd(w.dw + ((long long)co * 27 + tap) * w.cin + ci, acc[co]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kCols);
    }
    if (tid == 0 && (fail || !drained)) atomicExch(err, 1);
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
    int* d_err = nullptr;           // set by a tensor-core kernel whose mbarrier wait timed out (sticky)
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
void conv_launch(const tog_nn* nn, const ConvArgs& a, cudaStream_t s) {
    const long long M = a.dst.vox();
    const int grid = (int)((M + kTcRows - 1) / kTcRows);
    const size_t sm = conv_tc_smem(a.csrc, a.cdst);
    switch (a.cdst / 16) {
        case 1: k_conv_tc<TA, TO, 16, TR><<<grid, kTcRows, sm, s>>>(a, nn->d_err); break;
        case 2: k_conv_tc<TA, TO, 32, TR><<<grid, kTcRows, sm, s>>>(a, nn->d_err); break;
        case 3: k_conv_tc<TA, TO, 48, TR><<<grid, kTcRows, sm, s>>>(a, nn->d_err); break;
        default: k_conv_tc<TA, TO, 64, TR><<<grid, kTcRows, sm, s>>>(a, nn->d_err); break;
    }
}

// the tcgen05 kernels take more than the default 48 KB of dynamic shared memory
template <typename TA, typename TO, bool TR>
cudaError_t conv_tc_attributes() {
    const int sm = (int)conv_tc_smem(64, 64);
    cudaError_t e = cudaFuncSetAttribute(k_conv_tc<TA, TO, 16, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_tc<TA, TO, 32, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_tc<TA, TO, 48, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_tc<TA, TO, 64, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    return e;
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
    conv_launch<bf16, TO, false>(nn, a, nn->stream);
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
    conv_launch<float, float, true>(nn, a, nn->stream);
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
    const int gx = (27 * C.cin + kTcRows - 1) / kTcRows;
    const long long want = std::max<long long>(1, (long long)nn->nsm * 4 / gx);
    w.chunk = std::max<long long>(kWgVox, ((M + want - 1) / want + kWgVox - 1) / kWgVox * kWgVox);
    dim3 grid(gx, (unsigned)((M + w.chunk - 1) / w.chunk));
    const size_t sm = wgrad_tc_smem(C.cout);
    switch (C.cout / 16) {
        case 1: k_wgrad_tc<16><<<grid, kTcRows, sm, nn->stream>>>(w, nn->d_err); break;
        case 2: k_wgrad_tc<32><<<grid, kTcRows, sm, nn->stream>>>(w, nn->d_err); break;
        case 3: k_wgrad_tc<48><<<grid, kTcRows, sm, nn->stream>>>(w, nn->d_err); break;
        default: k_wgrad_tc<64><<<grid, kTcRows, sm, nn->stream>>>(w, nn->d_err); break;
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

int nn_status(tog_nn* nn, cudaStream_t stream) {
    int flag = 0;
    NN_CUDA(cudaMemcpyAsync(&flag, nn->d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    NN_CUDA(cudaStreamSynchronize(stream));
    if (flag) return nn_fail(TOG_ERR_CUDA, "warm-start network: a tensor-core convolution timed out waiting for its MMAs");
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
    R(nalloc(nn, &nn->d_err, 1));
    if (rc == TOG_OK) {
        cudaError_t e = conv_tc_attributes<bf16, bf16, false>();
        if (e == cudaSuccess) e = conv_tc_attributes<bf16, float, false>();
        if (e == cudaSuccess) e = conv_tc_attributes<float, float, true>();
        const int wsm = (int)wgrad_tc_smem(64);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wgrad_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, wsm);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wgrad_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, wsm);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wgrad_tc<48>, cudaFuncAttributeMaxDynamicSharedMemorySize, wsm);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wgrad_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, wsm);
        if (e != cudaSuccess) rc = nn_fail(TOG_ERR_CUDA, std::string("tog_nn_create: ") + cudaGetErrorString(e));
    }
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
    if (e == cudaSuccess) e = cudaMemset(nn->d_err, 0, sizeof(int));
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
    const int rc = nn_forward_dev(nn, in_dev, out_dev, nn->stream);
    return rc != TOG_OK ? rc : nn_status(nn, nn->stream);
}

int tog_nn_gradients(tog_nn* nn, const float* in_dev, const float* target_dev, double* loss, float* grads) {
    if (!nn || !in_dev || !target_dev) return nn_fail(TOG_ERR_ARG, "null argument");
    forward(nn, in_dev);
    double l = 0.0;
    int rc = backward(nn, target_dev, &l);
    if (rc != TOG_OK) return rc;
    if ((rc = nn_status(nn, nn->stream)) != TOG_OK) return rc;
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
    return loss ? nn_status(nn, nn->stream) : TOG_OK;
}

}  // extern "C"
