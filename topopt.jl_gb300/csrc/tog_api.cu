// C-ABI implementation of libtopopt_gb300 (see include/topopt_gb300.h).
// One tog_handle = one structured problem resident in HBM: design, densities,
// element scales, PCG vectors, filter stencil and OC scratch.  The per-iteration
// host<->device traffic of the device-resident loop is a handful of scalars.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/topopt_gb300.h"
#include "tog_host.h"
#include "tog_nn.h"
#include "tog_kernels.cuh"
#include "tog_mv3.cuh"
#include "tog_march3.cuh"
#include "tog_filter.cuh"
#include "tog_mma.cuh"

using namespace tog;

namespace {

thread_local std::string g_err;
std::atomic<long long> g_launches{0};

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define TOG_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? TOG_ERR_OOM : TOG_ERR_CUDA,               \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

#define TOG_TRY(call)               \
    do {                            \
        int s_ = (call);            \
        if (s_ != TOG_OK) return s_; \
    } while (0)

#define TOG_LAUNCHED(n) g_launches.fetch_add((n), std::memory_order_relaxed)

constexpr int kEwThreads = 256;
constexpr int kOcMaxSteps = 100;
// Iterations per pass of a device loop's WHILE body.  Every pass of a conditional node
// costs about 3 us of scheduling, 5% of a 56 us PCG iteration at 160x80x80; a body of
// several iterations pays it once per pass.  Kernels that find the state done return at
// once, so a pass that ends early costs those launches only.
constexpr int kPcgUnroll = 16;
constexpr int kOcUnroll = 4;

}  // namespace

int tog::set_error(int code, const char* msg) { return fail(code, msg); }

struct tog_handle {
    // problem
    int dim = 3;
    int32_t nel[3] = {1, 1, 1};
    int nn[3] = {2, 2, 2};
    long long nnodes = 0, ncells = 0, ndofs = 0;
    double size[3] = {1, 1, 1};
    double E = 1, nu = 0.3, xmin = 1e-3, p = 1;
    int plane_stress = 0;
    double meandiag = 0;
    double fnorm2 = 0;
    Modal<double, 3> M3d{};
    Modal<float, 3> M3f{};
    Modal<double, 2> M2d{};
    Modal<float, 2> M2f{};
    std::vector<int32_t> node_dofs;   // internal index -> reference dof
    std::vector<int32_t> ref2int;     // reference dof -> internal index
    // device
    cudaStream_t own = nullptr, stream = nullptr;
    int nsm = 152;
    int* d_int2ref = nullptr;
    int* d_ref2int = nullptr;
    uint8_t* d_fixmask = nullptr;
    double* d_f = nullptr;
    double* d_vars = nullptr;
    double* d_e64 = nullptr;
    float* d_e32 = nullptr;
    double* d_dinv64 = nullptr;
    float* d_dinv32 = nullptr;
    double *d_u = nullptr, *d_r64 = nullptr, *d_p64[2] = {nullptr, nullptr}, *d_q64 = nullptr;
    float *d_x32 = nullptr, *d_r32 = nullptr, *d_p32[2] = {nullptr, nullptr}, *d_q32 = nullptr;
    char* d_vecpool = nullptr;    // backing store of the dof-sized vectors below
    double* d_tmp = nullptr;      // dof-sized staging
    double* d_tmp2 = nullptr;
    double* d_cell[6] = {};       // cell-sized scratch
    double* d_nodal = nullptr;    // node-sized scratch
    PcgState* d_st64 = nullptr;
    PcgState* d_st32 = nullptr;
    OcState* d_oc = nullptr;
    double* d_partials = nullptr;
    size_t npartials = 0;
    unsigned* d_cnt = nullptr;    // misc counters
    double* d_scalar = nullptr;   // misc results
    PcgState* h_st = nullptr;     // pinned, two states (the FP32-IR segment reads both at once)
    OcState* h_oc = nullptr;
    double* h_scalar = nullptr;
    // filter
    int* d_soff = nullptr;
    double* d_sw = nullptr;
    int S = 0;
    double* d_invW = nullptr;
    bool filter_ready = false;
    double rmin = 0;
    FiltBox fbox{};            // node-offset range of the stencil
    bool filt_fused = false;   // shared-memory stencil kernels (else the two-pass kernels)
    int filt_lz = 1;           // cell planes per z band of the fused kernels
    size_t filt_smem[2] = {0, 0};
    // state
    bool vars_dirty = true;
    bool u_valid = false;
    // SIMP loop
    int simp_filter = TOG_FILTER_NONE;
    double volfrac = 0.5, move = 0.2;
    double *d_x = nullptr, *d_xnew = nullptr, *d_dc = nullptr, *d_dv = nullptr, *d_w = nullptr, *d_grad = nullptr,
           *d_B = nullptr;
    bool simp_ready = false;
    // active-element mask (FixedElementProjectorFun): position of each cell in x_free,
    // -1 black, -2 white; null when every cell is free
    int* d_fpos = nullptr;
    long long nfree = 0;
    // MMA: state, asymptotes / history / coefficients (10 cell vectors), iteration count
    // multi-load compliance: per-column cell gradients, saved single-load rhs, host maps
    double* d_mlg = nullptr;
    long long mlg_cols = 0;
    double* d_fsave = nullptr;
    MmaState* d_mma = nullptr;
    MmaState* h_mma = nullptr;
    double* d_mma_buf = nullptr;
    int mma_k = 0;
    int simp_opt = TOG_OPT_OC;
    double mma_move = 0.5;
    cudaGraphExec_t g_mma = nullptr;
    // learned warm start (3D): network, previous-iteration state and recording hook
    tog_nn* net = nullptr;
    double* d_vars_prev = nullptr;   // physical densities of the previous design iteration
    double* d_uprev = nullptr;       // displacement before the solve
    double* d_du_last = nullptr;     // displacement change of the previous design iteration
    bool have_du = false;
    float* d_nn_in = nullptr;        // network input (nodes x 8)
    float* d_nn_out = nullptr;       // network output (nodes x 3)
    double* d_nn_sc = nullptr;       // max |u|, max |f|, step lengths along the two directions
    double* d_nn_part = nullptr;
    unsigned* d_nn_cnt = nullptr;
    bool have_prev = false;
    float *rec_in = nullptr, *rec_tgt = nullptr;
    int rec_written = 0;
    // 3D operator tiling: tiles of 32 x MV3_BY elements, LZ layers per z chunk
    int nt[3] = {1, 1, 1};
    int LZ = 8;
    int march_grid = 0;        // persistent grid of k_march3 (the 3D FP32 PCG operator)
    int march_nband = 1, march_lzb = 1;   // its z bands per node column and their height
    double ru_delta = 0.03;    // FP32-IR reliable-update trigger: residual reduction factor (TOG_RU_DELTA)
    double* d_side64[8] = {};
    // graphs
    cudaGraphExec_t g_pcg64 = nullptr, g_pcg32 = nullptr, g_oc = nullptr;
    cudaGraphExec_t g_pcg64e = nullptr;   // FP64 batch with the EnergyCriteria check
    int conv = TOG_CONV_DEFAULT;
    int graph_nodes64 = 0, graph_nodes32 = 0;   // kernels per PCG iteration in the loop body
    int pcg_unroll = kPcgUnroll;                 // PCG iterations per pass of the body (TOG_PCG_UNROLL)

    Dims dims() const {
        Dims D;
        D.dim = dim;
        for (int d = 0; d < 3; ++d) {
            D.nel[d] = d < dim ? nel[d] : 1;
            D.nn[d] = d < dim ? nn[d] : 1;
        }
        D.nnodes = nnodes;
        D.ncells = ncells;
        return D;
    }
    int upd_per_sm = 2;        // PCG update blocks per SM (TOG_UPD_BLOCKS_PER_SM; 2 measured fastest)
    int upd_blocks() const {   // PCG update grid: a few blocks per SM, grid-stride over dof groups
        long long b = (3 * nnodes + 4LL * kEwThreads - 1) / (4LL * kEwThreads);
        const long long cap = (long long)nsm * upd_per_sm;   // the last-block reduction tail grows with the grid
        return (int)std::max(1LL, std::min(b, cap));
    }
    int ew_blocks(long long n) const {
        long long b = (n + kEwThreads - 1) / kEwThreads;
        long long cap = (long long)nsm * 8;
        if (b > cap) b = cap;
        if (b < 1) b = 1;
        return (int)b;
    }
};

namespace {

template <typename T>
int dalloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T) + 16);
    if (e != cudaSuccess) return fail(TOG_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return TOG_OK;
}

// Dof-sized vectors are read together at the same index; their base addresses
// are staggered by distinct multiples of 1.25 KiB inside one pool so that
// equal offsets do not land on the same DRAM channel.
template <typename T>
T* pool_take(char*& cursor, size_t n, int slot) {
    const size_t stagger = (size_t)slot * 1280;
    T* p = reinterpret_cast<T*>(cursor + stagger);
    const size_t bytes = ((n * sizeof(T) + stagger + 256 + 4095) / 4096) * 4096;
    cursor += bytes;
    return p;
}

dim3 mv3_grid(const tog_handle* h) {
    return dim3((h->nn[0] + 30) / 31, (h->nn[1] + MV_BY - 2) / (MV_BY - 1), (h->nn[2] + MV_LZ - 1) / MV_LZ);
}
dim3 mv2_grid(const tog_handle* h) {
    const int chunks = (h->nn[1] + MV2_LY - 1) / MV2_LY;
    return dim3((h->nn[0] + 30) / 31, (chunks + MV2_WARPS - 1) / MV2_WARPS, 1);
}

template <typename T>
MvArgs<T, 3> mv_args3(tog_handle* h);
template <>
MvArgs<double, 3> mv_args3<double>(tog_handle* h) {
    MvArgs<double, 3> A{};
    A.escale = h->d_e64;
    A.dinv = h->d_dinv64;
    A.r = h->d_r64;
    A.P0 = h->d_p64[0];
    A.P1 = h->d_p64[1];
    A.q = h->d_q64;
    A.st = h->d_st64;
    A.M = h->M3d;
    return A;
}
template <>
MvArgs<float, 3> mv_args3<float>(tog_handle* h) {
    MvArgs<float, 3> A{};
    A.escale = h->d_e32;
    A.dinv = h->d_dinv32;
    A.r = h->d_r32;
    A.P0 = h->d_p32[0];
    A.P1 = h->d_p32[1];
    A.q = h->d_q32;
    A.st = h->d_st32;
    A.M = h->M3f;
    return A;
}
template <typename T>
MvArgs<T, 2> mv_args2(tog_handle* h);
template <>
MvArgs<double, 2> mv_args2<double>(tog_handle* h) {
    MvArgs<double, 2> A{};
    A.escale = h->d_e64;
    A.dinv = h->d_dinv64;
    A.r = h->d_r64;
    A.P0 = h->d_p64[0];
    A.P1 = h->d_p64[1];
    A.q = h->d_q64;
    A.st = h->d_st64;
    A.M = h->M2d;
    return A;
}
template <>
MvArgs<float, 2> mv_args2<float>(tog_handle* h) {
    MvArgs<float, 2> A{};
    A.escale = h->d_e32;
    A.dinv = h->d_dinv32;
    A.r = h->d_r32;
    A.P0 = h->d_p32[0];
    A.P1 = h->d_p32[1];
    A.q = h->d_q32;
    A.st = h->d_st32;
    A.M = h->M2f;
    return A;
}

template <typename T, int DIM>
void fill_common(tog_handle* h, MvArgs<T, DIM>& A) {
    A.fixmask = h->d_fixmask;
    A.meandiag = (T)h->meandiag;
    for (int d = 0; d < 3; ++d) {
        A.nel[d] = d < h->dim ? h->nel[d] : 1;
        A.nn[d] = d < h->dim ? h->nn[d] : 1;
    }
    A.partials = h->d_partials;
}

template <typename T>
Mv3Args<T> mv3_args(tog_handle* h) {
    Mv3Args<T> A{};
    const MvArgs<T, 3> B = mv_args3<T>(h);
    A.r = B.r;
    A.P0 = B.P0;
    A.P1 = B.P1;
    A.q = B.q;
    A.escale = B.escale;
    A.dinv = B.dinv;
    A.st = B.st;
    A.M = B.M;
    A.fixmask = h->d_fixmask;
    A.partials = h->d_partials;
    for (int d = 0; d < 3; ++d) {
        A.nel[d] = h->nel[d];
        A.nn[d] = h->nn[d];
        A.nt[d] = h->nt[d];
    }
    A.LZ = h->LZ;
    A.div_nnx = make_fastdiv((unsigned)h->nn[0]);
    A.div_nny = make_fastdiv((unsigned)h->nn[1]);
    A.div_nnz = make_fastdiv((unsigned)h->nn[2]);
    for (int c = 0; c < 8; ++c)
        A.side[c] = std::is_same<T, double>::value ? (T*)h->d_side64[c] : nullptr;   // FP64 tile operator only
    return A;
}

template <typename T, int MODE>
void launch_mv3(tog_handle* h, cudaStream_t s, const Mv3Args<T>& A) {
    static bool attr_set = false;
    const int smem = (int)sizeof(Mv3Smem<T>);
    if (!attr_set) {
        cudaFuncSetAttribute(k_mv3<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set = true;
    }
    k_mv3<T, MODE><<<dim3(h->nt[0], h->nt[1], h->nt[2]), dim3(32, MV3_BY), smem, s>>>(A);
}

// Launch one matrix-free operator kernel (mode MV_*) in precision T.  3D PLAIN and
// RESID add the finalize kernel that gathers the tile-boundary partials.
template <typename T, int MODE>
void launch_matvec(tog_handle* h, cudaStream_t s, const T* x, T* y, const double* f) {
    if (h->dim == 3) {
        Mv3Args<T> A = mv3_args<T>(h);
        A.x = x;
        if (MODE == MV_RESID) A.st = h->d_st64;
        if constexpr (std::is_same<T, float>::value) {
            // FP32 is used by the PCG of the refinement only: the warp march
            static_assert(MODE == MV_PCG, "the 3D FP32 operator exists in PCG form only");
            k_march3<<<h->march_grid, 32 * kM3Warps, 0, s>>>(*reinterpret_cast<const Mv3Args<float>*>(&A),
                                                            (h->nn[0] + 29) / 30, h->march_nband, h->march_lzb);
        } else {
            launch_mv3<T, MODE>(h, s, A);
        }
        if constexpr (MODE != MV_PCG) {
            k_mv3_finalize<T, MODE><<<h->ew_blocks(h->nnodes), kEwThreads, 0, s>>>(A, x, y, f, (T)h->meandiag);
            TOG_LAUNCHED(1);
        }
    } else {
        MvArgs<T, 2> A = mv_args2<T>(h);
        fill_common<T, 2>(h, A);
        A.x = x;
        A.y = y;
        A.f = f;
        if (MODE == MV_RESID) A.st = h->d_st64;
        k_matvec2<T, MODE><<<mv2_grid(h), dim3(32, MV2_WARPS), 0, s>>>(A);
    }
    TOG_LAUNCHED(1);
}

template <typename T>
void launch_pcg_update(tog_handle* h, cudaStream_t s, LoopCond cond = LoopCond{}) {
    const int nb = h->ew_blocks(h->nnodes);
    if (h->dim == 3) {
        Mv3Args<T> A = mv3_args<T>(h);
        T* x = std::is_same<T, double>::value ? (T*)h->d_u : (T*)h->d_x32;
        T* r = std::is_same<T, double>::value ? (T*)h->d_r64 : (T*)h->d_r32;
        const long long n_side = (long long)(h->nt[0] - 1) * h->nn[1] * h->nn[2] +
                                 (long long)(h->nt[1] - 1) * h->nn[0] * h->nn[2] +
                                 (long long)(h->nt[2] - 1) * h->nn[0] * h->nn[1];
        // the FP32 march writes complete q: no tile-boundary partials to gather
        const bool march = std::is_same<T, float>::value;
        if (n_side > 0 && !march) {
            const long long nbs = std::min<long long>((n_side + kEwThreads - 1) / kEwThreads, (long long)h->nsm * 8);
            k_side_gather3<T><<<(int)nbs, kEwThreads, 0, s>>>(A);
            TOG_LAUNCHED(1);
        }
        // FP32: four float4 groups in flight per thread (53.4 against 54.1 us per PCG iteration
        // with two at 160x80x80)
        if (march)
            k_pcg_update3<T, 4><<<h->upd_blocks(), kEwThreads, 0, s>>>(A, x, r, (T)h->meandiag, cond);
        else
            k_pcg_update3<T><<<h->upd_blocks(), kEwThreads, 0, s>>>(A, x, r, (T)h->meandiag, cond);
    } else if (std::is_same<T, double>::value) {
            k_pcg_update<double, 2><<<nb, kEwThreads, 0, s>>>(h->d_u, h->d_r64, h->d_p64[0], h->d_p64[1], h->d_q64,
                                                              h->d_dinv64, h->M2d, h->nnodes, h->d_st64,
                                                              h->d_partials, cond);
    } else {
            k_pcg_update<float, 2><<<nb, kEwThreads, 0, s>>>(h->d_x32, h->d_r32, h->d_p32[0], h->d_p32[1], h->d_q32,
                                                             h->d_dinv32, h->M2f, h->nnodes, h->d_st32,
                                                             h->d_partials, cond);
    }
    TOG_LAUNCHED(1);
}

template <typename T>
void launch_pcg_init(tog_handle* h, cudaStream_t s, int zero_x, double rtol, double abstol, double bnorm2, int maxit,
                     double ru_delta2 = 0.0) {
    const int nb = h->ew_blocks(h->nnodes);
    if (std::is_same<T, double>::value) {
        if (h->dim == 3)
            k_pcg_init<double, 3><<<nb, kEwThreads, 0, s>>>(h->d_u, h->d_r64, h->d_p64[0], h->d_p64[1], h->d_dinv64,
                                                            h->M3d, h->nnodes, zero_x, rtol, abstol, bnorm2, maxit,
                                                            h->d_st64, h->d_partials, ru_delta2);
        else
            k_pcg_init<double, 2><<<nb, kEwThreads, 0, s>>>(h->d_u, h->d_r64, h->d_p64[0], h->d_p64[1], h->d_dinv64,
                                                            h->M2d, h->nnodes, zero_x, rtol, abstol, bnorm2, maxit,
                                                            h->d_st64, h->d_partials, ru_delta2);
    } else {
        if (h->dim == 3)
            k_pcg_init<float, 3><<<nb, kEwThreads, 0, s>>>(h->d_x32, h->d_r32, h->d_p32[0], h->d_p32[1],
                                                           h->d_dinv32, h->M3f, h->nnodes, zero_x, rtol, abstol,
                                                           bnorm2, maxit, h->d_st32, h->d_partials, ru_delta2);
        else
            k_pcg_init<float, 2><<<nb, kEwThreads, 0, s>>>(h->d_x32, h->d_r32, h->d_p32[0], h->d_p32[1],
                                                           h->d_dinv32, h->M2f, h->nnodes, zero_x, rtol, abstol,
                                                           bnorm2, maxit, h->d_st32, h->d_partials, ru_delta2);
    }
    TOG_LAUNCHED(1);
}

// The PCG iterations of one solve segment as ONE graph launch: a conditional WHILE
// node whose body is the operator, the update (and the EnergyCriteria check).  A
// first kernel sets the condition from the state (nothing runs if it is already
// done); the update's last block clears it once the state is done (converged,
// maxiter, breakdown or a reliable-update pause), so the loop stops on the device
// with no operator or update launched after convergence.
__global__ void k_pcg_cond_init(const PcgState* __restrict__ st, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0) cudaGraphSetConditional(h, st->done ? 0u : 1u);
}

template <typename T>
int build_pcg_graph(tog_handle* h, cudaGraphExec_t* out, bool energy = false) {
    PcgState* d_st = std::is_same<T, double>::value ? h->d_st64 : h->d_st32;
    cudaGraph_t g = nullptr;
    TOG_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle ch;
    TOG_CUDA(cudaGraphConditionalHandleCreate(&ch, g, 0, cudaGraphCondAssignDefault));
    // the condition from the state
    cudaGraphNode_t init;
    {
        cudaKernelNodeParams kp{};
        void* args[2] = {(void*)&d_st, (void*)&ch};
        kp.func = (void*)k_pcg_cond_init;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(32);
        kp.kernelParams = args;
        TOG_CUDA(cudaGraphAddKernelNode(&init, g, nullptr, 0, &kp));
    }
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = ch;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    TOG_CUDA(cudaGraphAddNode(&loop, g, &init, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    TOG_CUDA(cudaStreamBeginCaptureToGraph(h->own, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const long long before = g_launches.load();
    const int U = h->pcg_unroll;
    for (int k = 0; k < U; ++k) {   // only the body's last update sets the loop condition
        launch_matvec<T, MV_PCG>(h, h->own, nullptr, nullptr, nullptr);
        launch_pcg_update<T>(h, h->own, LoopCond{ch, k == U - 1 ? 1 : 0});
        if (energy) {
            k_energy_check<<<h->ew_blocks(h->ndofs), kEwThreads, 0, h->own>>>(h->d_u, h->d_r64, h->d_f, h->ndofs,
                                                                             h->d_st64, h->d_partials);
            TOG_LAUNCHED(1);
        }
    }
    // kernels per iteration; captured launches run only when the graph is launched
    const long long captured = g_launches.load() - before;
    g_launches.fetch_sub(captured);
    const int nodes = (int)(captured / U);
    (std::is_same<T, double>::value ? h->graph_nodes64 : h->graph_nodes32) = nodes;
    cudaGraph_t cap = nullptr;
    TOG_CUDA(cudaStreamEndCapture(h->own, &cap));
    TOG_CUDA(cudaGraphInstantiate(out, g, 0));
    cudaGraphDestroy(g);
    return TOG_OK;
}

int sync_state(tog_handle* h, const PcgState* d_st) {
    TOG_CUDA(cudaMemcpyAsync(h->h_st, d_st, sizeof(PcgState), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

// Launch the PCG iterations of the current state (to done) as one graph launch, without
// a host synchronisation.  A state that is already done runs no iteration: the graph's
// condition kernel sees it.
template <typename T>
int launch_pcg_loop(tog_handle* h, bool energy = false) {
    cudaGraphExec_t* g = std::is_same<T, double>::value ? (energy ? &h->g_pcg64e : &h->g_pcg64) : &h->g_pcg32;
    if (!*g) TOG_TRY(build_pcg_graph<T>(h, g, energy));
    TOG_CUDA(cudaGraphLaunch(*g, h->stream));
    return TOG_OK;
}

// Kernels of one launch_pcg_loop that took the state from iteration it0 to it1: the
// condition kernel and every pass of the body (the last one may end early: its remaining
// kernels find the state done and return; one more pass when an EnergyCriteria check
// ended the loop after the body's last update).
template <typename T>
void count_pcg_loop(tog_handle* h, int it0, int it1, bool energy = false) {
    if (it1 <= it0 && !energy) {
        TOG_LAUNCHED(1);
        return;
    }
    const long long passes = (it1 - it0 + h->pcg_unroll - 1) / h->pcg_unroll + (energy ? 1 : 0);
    TOG_LAUNCHED(1 + std::max(1LL, passes) * h->pcg_unroll *
                         (std::is_same<T, double>::value ? h->graph_nodes64 : h->graph_nodes32));
}

// Run the PCG iterations of the current state to done: one graph launch and one host
// synchronisation (plus one before, for the starting iteration count).
template <typename T>
int run_pcg(tog_handle* h, bool energy = false) {
    PcgState* d_st = std::is_same<T, double>::value ? h->d_st64 : h->d_st32;
    TOG_TRY(sync_state(h, d_st));
    const int it0 = h->h_st->it;
    if (h->h_st->done) return TOG_OK;
    TOG_TRY(launch_pcg_loop<T>(h, energy));
    TOG_TRY(sync_state(h, d_st));
    count_pcg_loop<T>(h, it0, h->h_st->it, energy);
    return TOG_OK;
}

int refresh_scales(tog_handle* h) {
    if (!h->vars_dirty) return TOG_OK;
    double ip_f = std::floor(h->p);
    const int ip = (h->p == ip_f && h->p >= 0 && h->p <= 8) ? (int)ip_f : -1;
    k_escale<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_vars, h->d_e64, h->d_e32, h->ncells,
                                                                   h->xmin, h->p, ip);
    TOG_LAUNCHED(1);
    if (h->dim == 3)
        k_nodesum<3><<<h->ew_blocks(h->nnodes), kEwThreads, 0, h->stream>>>(h->d_e64, h->d_dinv64, h->d_dinv32,
                                                                            h->dims());
    else
        k_nodesum<2><<<h->ew_blocks(h->nnodes), kEwThreads, 0, h->stream>>>(h->d_e64, h->d_dinv64, h->d_dinv32,
                                                                            h->dims());
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    h->vars_dirty = false;
    return TOG_OK;
}

int solve_fp64(tog_handle* h, double rtol, double abstol, int maxit, int warm, tog_solve_stats* st) {
    if (warm && h->u_valid) {
        launch_matvec<double, MV_RESID>(h, h->stream, h->d_u, h->d_r64, h->d_f);
        launch_pcg_init<double>(h, h->stream, 0, rtol, abstol, h->fnorm2, maxit);
    } else {
        TOG_CUDA(cudaMemcpyAsync(h->d_r64, h->d_f, h->ndofs * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
        launch_pcg_init<double>(h, h->stream, 1, rtol, abstol, h->fnorm2, maxit);
    }
    const bool energy = h->conv == TOG_CONV_ENERGY;
    if (energy) {   // the stop rule of EnergyCriteria, first checked on the start vector
        k_energy_init<<<1, 32, 0, h->stream>>>(h->d_st64);
        k_energy_check<<<h->ew_blocks(h->ndofs), kEwThreads, 0, h->stream>>>(h->d_u, h->d_r64, h->d_f, h->ndofs,
                                                                            h->d_st64, h->d_partials);
        TOG_LAUNCHED(2);
    }
    TOG_CUDA(cudaGetLastError());
    TOG_TRY(run_pcg<double>(h, energy));
    h->u_valid = true;
    const PcgState& s = *h->h_st;
    if (st) {
        st->status = s.status;
        st->iterations = s.it;
        st->outer_iterations = 0;
        st->abs_residual = std::sqrt(s.rr);
        st->rel_residual = h->fnorm2 > 0 ? std::sqrt(s.rr / h->fnorm2) : std::sqrt(s.rr);
    }
    if (s.status == 7)
        return fail(TOG_BREAKDOWN, "EnergyCriteria: NaN or negative x'Ax (the reference's DomainError)");
    return s.status == 0 ? TOG_OK : fail(s.status, s.status == 3 ? "PCG did not converge within maxiter"
                                                                   : "PCG breakdown (p'Kp <= 0 or NaN)");
}

// FP32 PCG inside FP64 refinement with reliable updates: the FP32 iteration
// pauses whenever its residual has dropped by ru_delta since the last update
// (or looks converged); the host then folds x32 into the FP64 solution,
// recomputes the FP64 true residual and rescales the FP32 state, keeping the
// search direction, so the Krylov progress is not thrown away as by a restart.
int solve_fp32_ir(tog_handle* h, double rtol, double abstol, int maxit, int warm, tog_solve_stats* st) {
    const long long nd = h->ndofs;
    if (!(warm && h->u_valid)) TOG_CUDA(cudaMemsetAsync(h->d_u, 0, nd * sizeof(double), h->stream));
    const double tol = std::fmax(rtol * std::sqrt(h->fnorm2), abstol);
    const int nb = h->ew_blocks(nd);
    auto resid = [&](double* res) -> int {
        launch_matvec<double, MV_RESID>(h, h->stream, h->d_u, h->d_r64, h->d_f);
        TOG_CUDA(cudaGetLastError());
        TOG_TRY(sync_state(h, h->d_st64));
        *res = std::sqrt(h->h_st->rr);
        return TOG_OK;
    };
    int status = TOG_OK, updates = 0, inner = 0;
    double res = 0.0;
    TOG_TRY(resid(&res));
    if (std::isfinite(res) && res > tol) {
        double s = res;
        if (h->dim == 3)
            k_ir_scale<3><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, nd, h->d_st64);
        else
            k_ir_scale<2><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, nd, h->d_st64);
        TOG_LAUNCHED(1);
        launch_pcg_init<float>(h, h->stream, 1, 0.0, tol / s, -1.0, maxit, h->ru_delta * h->ru_delta);
        TOG_CUDA(cudaGetLastError());
        double best = res;
        int since_best = 0;
        int it0 = 0;   // FP32 iteration count at the start of the segment
        for (;;) {
            // one segment: the FP32 PCG loop, the fold into u and the FP64 true residual,
            // then one host synchronisation for both states
            TOG_TRY(launch_pcg_loop<float>(h));
            k_ir_correct<<<nb, kEwThreads, 0, h->stream>>>(h->d_u, h->d_x32, nd, s);
            TOG_LAUNCHED(1);
            launch_matvec<double, MV_RESID>(h, h->stream, h->d_u, h->d_r64, h->d_f);
            TOG_CUDA(cudaGetLastError());
            TOG_CUDA(cudaMemcpyAsync(h->h_st, h->d_st32, sizeof(PcgState), cudaMemcpyDeviceToHost, h->stream));
            TOG_CUDA(cudaMemcpyAsync(h->h_st + 1, h->d_st64, sizeof(PcgState), cudaMemcpyDeviceToHost, h->stream));
            TOG_CUDA(cudaStreamSynchronize(h->stream));
            const PcgState s32 = h->h_st[0];
            count_pcg_loop<float>(h, it0, s32.it);
            inner = s32.it;
            it0 = s32.it;
            res = std::sqrt(h->h_st[1].rr);
            ++updates;
            if (!std::isfinite(res)) {
                status = TOG_BREAKDOWN;
                break;
            }
            if (res <= tol) break;
            if (res < 0.5 * best) {
                best = res;
                since_best = 0;
            } else if (++since_best >= 8) {   // FP64 residual stalled above tol
                status = TOG_NOT_CONVERGED;
                break;
            }
            if (s32.status == 3 || inner >= maxit) {
                status = TOG_NOT_CONVERGED;
                break;
            }
            if (s32.status == 4) {
                // breakdown of the FP32 recurrence: restart from the true residual
                if (h->dim == 3)
                    k_ir_scale<3><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, nd, h->d_st64);
                else
                    k_ir_scale<2><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, nd, h->d_st64);
                TOG_LAUNCHED(1);
                launch_pcg_init<float>(h, h->stream, 1, 0.0, tol / res, -1.0, maxit - inner,
                                       h->ru_delta * h->ru_delta);
                s = res;
                it0 = 0;
                continue;
            }
            const double t2 = (tol / res) * (tol / res);
            if (h->dim == 3)
                k_ru_rescale<3><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, h->d_x32, h->d_p32[0],
                                                                  h->d_p32[1], h->d_dinv32, h->M3f, h->nnodes, s,
                                                                  res, t2, h->d_st32, h->d_partials);
            else
                k_ru_rescale<2><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, h->d_x32, h->d_p32[0],
                                                                  h->d_p32[1], h->d_dinv32, h->M2f, h->nnodes, s,
                                                                  res, t2, h->d_st32, h->d_partials);
            TOG_LAUNCHED(1);
            TOG_CUDA(cudaGetLastError());
            s = res;
        }
    }
    h->u_valid = true;
    if (st) {
        st->status = status;
        st->iterations = inner;
        st->outer_iterations = updates;
        st->abs_residual = res;
        st->rel_residual = h->fnorm2 > 0 ? res / std::sqrt(h->fnorm2) : res;
    }
    if (status != TOG_OK) {
        char msg[200];
        std::snprintf(msg, sizeof msg, "FP32-IR %s: ||f-Ku||/||f|| = %.3e after %d PCG iterations, %d updates",
                      status == TOG_BREAKDOWN ? "breakdown" : "did not reach the FP64 tolerance",
                      h->fnorm2 > 0 ? res / std::sqrt(h->fnorm2) : res, inner, updates);
        return fail(status, msg);
    }
    return TOG_OK;
}

// ---------------------------------------------------------------------------
// learned warm start (3D structured grids; no counterpart in TopOpt.jl)
// ---------------------------------------------------------------------------
constexpr int kNnBlocks = 1024;   // grid of the warm-start reductions (partials sized for it)

// sc[0] = max |u| (1 when zero), sc[1] = max |r0| (1 when zero)
__global__ void k_nn_scales(const double* __restrict__ u, const double* __restrict__ f, long long n,
                            double* partials, unsigned* cnt, double* sc) {
    double v[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        v[0] = fmax(v[0], fabs(u[i]));
        v[1] = fmax(v[1], fabs(f[i]));
    }
    double tot[2];
    if (grid_reduce_last<2, true>(v, partials, cnt, tot) && threadIdx.x == 0) {
        sc[0] = tot[0] > 0.0 ? tot[0] : 1.0;
        sc[1] = tot[1] > 0.0 ? tot[1] : 1.0;
    }
}

// network input per node: mean of the adjacent cells' new physical density and of
// its change, u / max|u| and the residual r0 = f - K(rho_new) u over max|r0|
// (internal AoS dof layout 3 n + c).  The target, the solve's correction, is
// K^-1 r0: the network learns an approximate inverse of K(rho) applied to r0.
__global__ void k_nn_input(Dims D, const double* __restrict__ vars, const double* __restrict__ prev,
                           const double* __restrict__ u, const double* __restrict__ f, const double* __restrict__ sc,
                           float* __restrict__ out) {
    const double iu = 1.0 / sc[0], iff = 1.0 / sc[1];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < D.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(n % D.nn[0]), iy = (int)((n / D.nn[0]) % D.nn[1]), iz = (int)(n / ((long long)D.nn[0] * D.nn[1]));
        double s = 0.0, ds = 0.0;
        int c = 0;
        for (int dz = -1; dz <= 0; ++dz)
            for (int dy = -1; dy <= 0; ++dy)
                for (int dx = -1; dx <= 0; ++dx) {
                    const int cx = ix + dx, cy = iy + dy, cz = iz + dz;
                    if (cx < 0 || cy < 0 || cz < 0 || cx >= D.nel[0] || cy >= D.nel[1] || cz >= D.nel[2]) continue;
                    const long long e = cx + (long long)D.nel[0] * (cy + (long long)D.nel[1] * cz);
                    s += vars[e];
                    ds += vars[e] - prev[e];
                    ++c;
                }
        float* o = out + 8 * n;
        o[0] = (float)(s / c);
        o[1] = (float)(ds / c);
        for (int k = 0; k < 3; ++k) {
            o[2 + k] = (float)(u[3 * n + k] * iu);
            o[5 + k] = (float)(f[3 * n + k] * iff);
        }
    }
}

// correction direction d = network output (trained on the density-weighted
// correction rho~ (u_new - u_prev): in near-void regions the displacement is barely
// constrained and a guess there only adds work for PCG), zero at fixed dofs
__global__ void k_nn_direction(const float* __restrict__ y, const uint8_t* __restrict__ fixmask,
                               double* __restrict__ d, long long nnodes) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 3 * nnodes;
         i += (long long)gridDim.x * blockDim.x) {
        const long long n = i / 3;
        const int c = (int)(i - 3 * n);
        d[i] = ((fixmask[n] >> c) & 1u) ? 0.0 : (double)y[i];
    }
}

// Galerkin step on span{d1, d2} (d2 may be absent): minimise the energy norm of the
// error, i.e. solve [d1.Kd1 d1.Kd2; d2.Kd1 d2.Kd2] c = [d1.r0; d2.r0] with r0 = f - K u.
// A singular or indefinite 2 x 2 system falls back to the better single direction;
// a direction with d.Kd <= 0 gets no step.  c -> sc[2], sc[3].
__global__ void k_nn_galerkin(const double* __restrict__ d1, const double* __restrict__ kd1,
                              const double* __restrict__ d2, const double* __restrict__ kd2,
                              const double* __restrict__ r0, long long n, double* partials, unsigned* cnt,
                              double* sc) {
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double a = d1 ? d1[i] : 0.0, b = d2 ? d2[i] : 0.0;
        v[0] = fma(a, kd1 ? kd1[i] : 0.0, v[0]);   // d1.Kd1
        v[1] = fma(a, kd2 ? kd2[i] : 0.0, v[1]);   // d1.Kd2
        v[2] = fma(b, kd2 ? kd2[i] : 0.0, v[2]);   // d2.Kd2
        v[3] = fma(a, r0[i], v[3]);                 // d1.r0
        v[4] = fma(b, r0[i], v[4]);                 // d2.r0
    }
    double t[5];
    if (grid_reduce_last<5>(v, partials, cnt, t) && threadIdx.x == 0) {
        const double a11 = t[0], a12 = t[1], a22 = t[2], b1 = t[3], b2 = t[4];
        double c1 = a11 > 0.0 ? b1 / a11 : 0.0, c2 = a22 > 0.0 ? b2 / a22 : 0.0;
        // energy decrease of each single direction: b^2 / a
        const double g1 = a11 > 0.0 ? b1 * c1 : 0.0, g2 = a22 > 0.0 ? b2 * c2 : 0.0;
        const double det = a11 * a22 - a12 * a12;
        if (a11 > 0.0 && a22 > 0.0 && det > 1e-10 * a11 * a22) {
            c1 = (b1 * a22 - b2 * a12) / det;
            c2 = (b2 * a11 - b1 * a12) / det;
        } else if (g1 >= g2) {
            c2 = 0.0;
        } else {
            c1 = 0.0;
        }
        sc[2] = isfinite(c1) ? c1 : 0.0;
        sc[3] = isfinite(c2) ? c2 : 0.0;
    }
}

__global__ void k_nn_step(double* __restrict__ u, const double* __restrict__ d1, const double* __restrict__ d2,
                          const double* __restrict__ sc, long long n) {
    const double c1 = sc[2], c2 = sc[3];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        u[i] = fma(c1, d1 ? d1[i] : 0.0, fma(c2, d2 ? d2[i] : 0.0, u[i]));
}

__global__ void k_sub(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c[i] = a[i] - b[i];
}

// training target: (u_new - u_prev) / max|u_prev|
__global__ void k_nn_target(const double* __restrict__ u, const double* __restrict__ uprev,
                            const double* __restrict__ sc, float* __restrict__ tgt, long long n) {
    const double iu = 1.0 / sc[0];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        tgt[i] = (float)((u[i] - uprev[i]) * iu);
}

int nn_buffers(tog_handle* h) {
    if (h->d_vars_prev) return TOG_OK;
    int rc = TOG_OK;
    auto A = [&](int r) {
        if (rc == TOG_OK) rc = r;
    };
    A(dalloc(&h->d_vars_prev, h->ncells));
    A(dalloc(&h->d_uprev, h->ndofs));
    A(dalloc(&h->d_du_last, h->ndofs));
    A(dalloc(&h->d_nn_in, 8 * h->nnodes));
    A(dalloc(&h->d_nn_out, 3 * h->nnodes));
    A(dalloc(&h->d_nn_sc, 4));
    A(dalloc(&h->d_nn_part, 5 * kNnBlocks));
    A(dalloc(&h->d_nn_cnt, 4));
    if (rc != TOG_OK) return rc;
    TOG_CUDA(cudaMemsetAsync(h->d_nn_cnt, 0, 4 * sizeof(unsigned), h->stream));
    h->have_prev = false;
    h->have_du = false;
    return TOG_OK;
}

// Before the solve of a design iteration (new physical densities in d_vars, the
// previous solution in d_u): keep u_prev, write the network input (into the
// recording buffer when one is set) and, for the learned and extrapolated starts,
// move d_u by the Galerkin step on span{network correction, last change}
// (learned) or along the last change alone (extrapolated).  Either never increases
// the energy norm of the error.
int nn_before_solve(tog_handle* h, bool use_net, bool use_du) {
    cudaStream_t s = h->stream;
    const int nb = (int)std::min<long long>(kNnBlocks, h->ew_blocks(h->ndofs));
    TOG_CUDA(cudaMemcpyAsync(h->d_uprev, h->d_u, h->ndofs * sizeof(double), cudaMemcpyDeviceToDevice, s));
    use_du = use_du && h->have_du;
    const bool input = use_net || h->rec_in;
    if (!(input || use_du)) return TOG_OK;
    TOG_TRY(refresh_scales(h));
    launch_matvec<double, MV_RESID>(h, s, h->d_u, h->d_r64, h->d_f);   // r0 = f - K(rho_new) u
    float* in = nullptr;
    if (input) {
        k_nn_scales<<<nb, kEwThreads, 0, s>>>(h->d_u, h->d_r64, h->ndofs, h->d_nn_part, h->d_nn_cnt, h->d_nn_sc);
        in = h->rec_in ? h->rec_in : h->d_nn_in;
        k_nn_input<<<h->ew_blocks(h->nnodes), kEwThreads, 0, s>>>(h->dims(), h->d_vars, h->d_vars_prev, h->d_u,
                                                                 h->d_r64, h->d_nn_sc, in);
    }
    if (use_net || use_du) {
        double* d1 = nullptr;
        double* d2 = use_du ? h->d_du_last : nullptr;
        if (use_net) {
            TOG_TRY(nn_forward_dev(h->net, in, h->d_nn_out, s));
            k_nn_direction<<<h->ew_blocks(h->ndofs), kEwThreads, 0, s>>>(h->d_nn_out, h->d_fixmask, h->d_tmp,
                                                                       h->nnodes);
            d1 = h->d_tmp;
            launch_matvec<double, MV_PLAIN>(h, s, d1, h->d_q64, nullptr);          // K d1
        }
        if (d2) launch_matvec<double, MV_PLAIN>(h, s, d2, h->d_p64[1], nullptr);   // K d2
        k_nn_galerkin<<<nb, kEwThreads, 0, s>>>(d1, d1 ? h->d_q64 : nullptr, d2, d2 ? h->d_p64[1] : nullptr, h->d_r64,
                                                h->ndofs, h->d_nn_part, h->d_nn_cnt + 1, h->d_nn_sc);
        k_nn_step<<<h->ew_blocks(h->ndofs), kEwThreads, 0, s>>>(h->d_u, d1, d2, h->d_nn_sc, h->ndofs);
    }
    TOG_CUDA(cudaGetLastError());
    return TOG_OK;
}

// Projections of a density field and their derivatives (penalties.jl:75-96):
//   Heaviside (kind 1): y = 1 - exp(-beta x) + x exp(-beta), y' = beta exp(-beta x) + exp(-beta)
//   sigmoid   (kind 2): y = 1 / (1 + exp((beta + 1) (0.5 - x))), y' = (beta + 1) y (1 - y)
__global__ void k_projection(int kind, double beta, const double* __restrict__ x, double* __restrict__ y,
                             double* __restrict__ dy, long long n) {
    const double eb = exp(-beta);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double xi = x[i];
        if (kind == TOG_PROJ_HEAVISIDE) {
            const double e = exp(-beta * xi);
            y[i] = 1.0 - e + xi * eb;
            dy[i] = beta * e + eb;
        } else {
            const double s = 1.0 / (1.0 + exp((beta + 1.0) * (0.5 - xi)));
            y[i] = s;
            dy[i] = (beta + 1.0) * s * (1.0 - s);
        }
    }
}

int do_solve(tog_handle* h, int prec, double rtol, double abstol, int maxit, int warm, tog_solve_stats* st) {
    TOG_TRY(refresh_scales(h));
    if (prec == TOG_FP32_IR && h->conv == TOG_CONV_ENERGY)
        return fail(TOG_ERR_ARG, "EnergyCriteria is a stop rule of the FP64 solve (FP32-IR stops on the FP64 "
                                 "true residual)");
    if (prec == TOG_FP64) return solve_fp64(h, rtol, abstol, maxit, warm, st);
    if (prec == TOG_FP32_IR) return solve_fp32_ir(h, rtol, abstol, maxit, warm, st);
    return fail(TOG_ERR_ARG, "unknown precision");
}

int compliance_dev(tog_handle* h, double* d_grad) {
    const int nb = h->ew_blocks(h->ncells);
    double ip_f = std::floor(h->p);
    const int ip = (h->p == ip_f && h->p >= 0 && h->p <= 8) ? (int)ip_f : -1;
    if (h->dim == 3)
        k_compliance<3><<<nb, kEwThreads, 0, h->stream>>>(h->d_u, h->d_vars, h->M3d, h->xmin, h->p, ip, h->dims(),
                                                          d_grad, nullptr, h->d_partials, h->d_cnt, h->d_scalar);
    else
        k_compliance<2><<<nb, kEwThreads, 0, h->stream>>>(h->d_u, h->d_vars, h->M2d, h->xmin, h->p, ip, h->dims(),
                                                          d_grad, nullptr, h->d_partials, h->d_cnt, h->d_scalar);
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    return TOG_OK;
}

// y = J x (op 0) or J' x (op 1), device arrays
int filter_dev(tog_handle* h, int op, const double* in, double* out) {
    const Dims D = h->dims();
    const int nbn = h->ew_blocks(h->nnodes), nbc = h->ew_blocks(h->ncells);
    cudaStream_t s = h->stream;
    if (h->filt_fused) {
        const dim3 grid((D.nel[0] + kFiltTX - 1) / kFiltTX, (D.nel[1] + kFiltTY - 1) / kFiltTY,
                        h->dim == 3 ? (D.nel[2] + h->filt_lz - 1) / h->filt_lz : 1);
        const int nt = kFiltTX * kFiltTY;
        if (op == TOG_FILTER_J) {
            if (h->dim == 3)
                k_filt_fwd<3><<<grid, nt, h->filt_smem[0], s>>>(in, out, h->d_soff, h->d_sw, h->S, h->d_invW, D,
                                                                h->fbox, h->filt_lz);
            else
                k_filt_fwd<2><<<grid, nt, h->filt_smem[0], s>>>(in, out, h->d_soff, h->d_sw, h->S, h->d_invW, D,
                                                                h->fbox, 1);
        } else {
            if (h->dim == 3)
                k_filt_bwd<3><<<grid, nt, h->filt_smem[1], s>>>(in, out, h->d_soff, h->d_sw, h->S, h->d_invW, D,
                                                                h->fbox, h->filt_lz);
            else
                k_filt_bwd<2><<<grid, nt, h->filt_smem[1], s>>>(in, out, h->d_soff, h->d_sw, h->S, h->d_invW, D,
                                                                h->fbox, 1);
        }
        TOG_LAUNCHED(1);
        TOG_CUDA(cudaGetLastError());
        return TOG_OK;
    }
    if (op == TOG_FILTER_J) {
        if (h->dim == 3) {
            k_filt_node_avg<3><<<nbn, kEwThreads, 0, s>>>(in, h->d_nodal, D);
            k_filt_cone<3><<<nbc, kEwThreads, 0, s>>>(h->d_nodal, out, h->d_soff, h->d_sw, h->S, h->d_invW, in, D);
        } else {
            k_filt_node_avg<2><<<nbn, kEwThreads, 0, s>>>(in, h->d_nodal, D);
            k_filt_cone<2><<<nbc, kEwThreads, 0, s>>>(h->d_nodal, out, h->d_soff, h->d_sw, h->S, h->d_invW, in, D);
        }
    } else {
        if (h->dim == 3) {
            k_filt_cone_T<3><<<nbn, kEwThreads, 0, s>>>(in, h->d_nodal, h->d_soff, h->d_sw, h->S, h->d_invW, D);
            k_filt_node_avg_T<3><<<nbc, kEwThreads, 0, s>>>(h->d_nodal, out, D);
        } else {
            k_filt_cone_T<2><<<nbn, kEwThreads, 0, s>>>(in, h->d_nodal, h->d_soff, h->d_sw, h->S, h->d_invW, D);
            k_filt_node_avg_T<2><<<nbc, kEwThreads, 0, s>>>(h->d_nodal, out, D);
        }
    }
    TOG_LAUNCHED(2);
    TOG_CUDA(cudaGetLastError());
    return TOG_OK;
}

// The OC bisection as one graph: a conditional WHILE node over k_oc_step (whose last
// block stops the loop once the bisection has converged or run kOcMaxSteps steps), then
// the new design.
int build_oc_graph(tog_handle* h) {
    cudaGraph_t g = nullptr;
    TOG_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle ch;
    TOG_CUDA(cudaGraphConditionalHandleCreate(&ch, g, 0, cudaGraphCondAssignDefault));
    OcState* d_oc = h->d_oc;
    cudaGraphNode_t init;
    {
        cudaKernelNodeParams kp{};
        void* args[2] = {(void*)&d_oc, (void*)&ch};
        kp.func = (void*)k_oc_cond_init;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(32);
        kp.kernelParams = args;
        TOG_CUDA(cudaGraphAddKernelNode(&init, g, nullptr, 0, &kp));
    }
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = ch;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    TOG_CUDA(cudaGraphAddNode(&loop, g, &init, nullptr, 1, &cp));
    const int nb = h->ew_blocks(h->ncells);
    TOG_CUDA(cudaStreamBeginCaptureToGraph(h->own, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kOcUnroll; ++k)   // only the body's last step sets the loop condition
        k_oc_step<<<nb, kEwThreads, 0, h->own>>>(h->d_x, h->d_B, h->d_w, h->ncells, h->d_oc, h->d_partials,
                                                 h->d_fpos, LoopCond{ch, k == kOcUnroll - 1 ? 1 : 0});
    cudaGraph_t body = nullptr;
    TOG_CUDA(cudaStreamEndCapture(h->own, &body));
    TOG_CUDA(cudaStreamBeginCaptureToGraph(h->own, g, &loop, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    k_oc_final<<<nb, kEwThreads, 0, h->own>>>(h->d_x, h->d_B, h->d_xnew, h->ncells, h->d_oc, h->d_partials,
                                               h->d_w, h->d_fpos);
    cudaGraph_t cap = nullptr;
    TOG_CUDA(cudaStreamEndCapture(h->own, &cap));
    TOG_CUDA(cudaGraphInstantiate(&h->g_oc, g, 0));
    cudaGraphDestroy(g);
    return TOG_OK;
}

// OC on the device arrays d_x, d_dc, d_dv, d_w -> d_xnew
int oc_dev(tog_handle* h, double volfrac, double move) {
    if (!h->g_oc) TOG_TRY(build_oc_graph(h));
    const int nb = h->ew_blocks(h->ncells);
    k_oc_prep<<<nb, kEwThreads, 0, h->stream>>>(h->d_x, h->d_dc, h->d_dv, h->d_B, h->ncells, h->d_oc, 0.0, 1e9, 1e-3,
                                                volfrac, move, kOcMaxSteps);
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    TOG_CUDA(cudaGraphLaunch(h->g_oc, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->h_oc, h->d_oc, sizeof(OcState), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    // condition, every pass of the body (the last may end early), final
    TOG_LAUNCHED(2 + (long long)std::max(1, (h->h_oc->steps + kOcUnroll - 1) / kOcUnroll) * kOcUnroll);
    return TOG_OK;
}

MmaArgs mma_args(tog_handle* h, const double* w) {
    MmaArgs A{};
    const long long n = h->ncells;
    A.x = h->d_x;
    A.df0 = h->d_dc;
    A.dg = h->d_dv;
    A.w = w;
    A.fpos = h->d_fpos;
    double* b = h->d_mma_buf;
    A.low = b;
    A.upp = b + n;
    A.xold1 = b + 2 * n;
    A.xold2 = b + 3 * n;
    A.alfa = b + 4 * n;
    A.beta = b + 5 * n;
    A.p0 = b + 6 * n;
    A.q0 = b + 7 * n;
    A.p1 = b + 8 * n;
    A.q1 = b + 9 * n;
    A.xnew = h->d_xnew;
    A.n = n;
    A.st = h->d_mma;
    A.partials = h->d_partials;
    return A;
}

int mma_buffers(tog_handle* h) {
    if (h->d_mma) return TOG_OK;
    TOG_TRY(dalloc(&h->d_mma, 1));
    TOG_TRY(dalloc(&h->d_mma_buf, 10 * (size_t)h->ncells));
    TOG_CUDA(cudaMallocHost(&h->h_mma, sizeof(MmaState)));
    TOG_CUDA(cudaMemsetAsync(h->d_mma, 0, sizeof(MmaState), h->stream));
    return TOG_OK;
}

// One MMA update on the device arrays d_x, d_dc (objective gradient), d_dv (constraint
// gradient) -> d_xnew.  With use_w the constraint is sum(d_w x) - volfrac, else g.
int mma_dev(tog_handle* h, bool use_w, double g, double volfrac, double move) {
    TOG_TRY(mma_buffers(h));
    const int nb = h->ew_blocks(h->ncells);
    if (!h->g_mma) {
        cudaGraph_t gr = nullptr;
        const MmaArgs A = mma_args(h, h->d_w);
        TOG_CUDA(cudaStreamBeginCapture(h->own, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < kMmaMaxSteps; ++i) k_mma_step<<<nb, kEwThreads, 0, h->own>>>(A);
        k_mma_final<<<nb, kEwThreads, 0, h->own>>>(A);
        TOG_CUDA(cudaStreamEndCapture(h->own, &gr));
        TOG_CUDA(cudaGraphInstantiate(&h->g_mma, gr, 0));
        cudaGraphDestroy(gr);
    }
    h->mma_k += 1;
    k_mma_prep<<<nb, kEwThreads, 0, h->stream>>>(mma_args(h, use_w ? h->d_w : nullptr), h->mma_k, g, volfrac,
                                                 move);
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    TOG_CUDA(cudaGraphLaunch(h->g_mma, h->stream));
    TOG_LAUNCHED(kMmaMaxSteps + 1);
    TOG_CUDA(cudaMemcpyAsync(h->h_mma, h->d_mma, sizeof(MmaState), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int upload_dofs(tog_handle* h, const double* ref, double* d_internal) {
    TOG_CUDA(cudaMemcpyAsync(h->d_tmp2, ref, h->ndofs * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    k_gather_d<<<h->ew_blocks(h->ndofs), kEwThreads, 0, h->stream>>>(h->d_tmp2, h->d_int2ref, d_internal, h->ndofs);
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    return TOG_OK;
}
int download_dofs(tog_handle* h, const double* d_internal, double* ref) {
    k_gather_d<<<h->ew_blocks(h->ndofs), kEwThreads, 0, h->stream>>>(d_internal, h->d_ref2int, h->d_tmp2, h->ndofs);
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    TOG_CUDA(cudaMemcpyAsync(ref, h->d_tmp2, h->ndofs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int check_handle(tog_handle* h) {
    if (!h) return fail(TOG_ERR_ARG, "null handle");
    return TOG_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char* tog_version(void) { return "libtopopt_gb300 1 (sm_103a)"; }
const char* tog_last_error(void) { return g_err.c_str(); }
int64_t tog_launch_count(void) { return g_launches.load(); }

int tog_grid_counts(int32_t dim, const int32_t* nel, int64_t* nnodes, int64_t* ncells, int64_t* ndofs) {
    if ((dim != 2 && dim != 3) || !nel) return fail(TOG_ERR_ARG, "dim must be 2 or 3");
    for (int d = 0; d < dim; ++d)
        if (nel[d] < 1) return fail(TOG_ERR_ARG, "nel must be >= 1");
    long long nn, nc;
    grid_counts(dim, nel, &nn, &nc);
    if (nnodes) *nnodes = nn;
    if (ncells) *ncells = nc;
    if (ndofs) *ndofs = nn * dim;
    return TOG_OK;
}

int tog_node_dofs(int32_t dim, const int32_t* nel, int32_t* node_dofs) {
    TOG_TRY(tog_grid_counts(dim, nel, nullptr, nullptr, nullptr));
    if (!node_dofs) return fail(TOG_ERR_ARG, "null output");
    node_dofs_first_touch(dim, nel, node_dofs);
    return TOG_OK;
}

int tog_cell_dofs(int32_t dim, const int32_t* nel, int32_t* cell_dofs) {
    int64_t nn;
    TOG_TRY(tog_grid_counts(dim, nel, &nn, nullptr, nullptr));
    if (!cell_dofs) return fail(TOG_ERR_ARG, "null output");
    std::vector<int32_t> nd((size_t)nn * dim);
    node_dofs_first_touch(dim, nel, nd.data());
    cell_dofs_from_node_dofs(dim, nel, nd.data(), cell_dofs);
    return TOG_OK;
}

int tog_element_stiffness(int32_t dim, const double* size, double E, double nu, int32_t plane_stress, double* Ke) {
    if ((dim != 2 && dim != 3) || !size || !Ke) return fail(TOG_ERR_ARG, "bad arguments");
    if (!(nu > -1.0 && nu < 0.5) || !(E > 0)) return fail(TOG_ERR_ARG, "need E > 0 and -1 < nu < 0.5");
    element_stiffness(dim, size, E, nu, plane_stress, Ke);
    return TOG_OK;
}

int tog_create(const tog_problem_desc* desc, tog_handle** out) {
    if (!desc || !out) return fail(TOG_ERR_ARG, "null argument");
    *out = nullptr;
    const int dim = desc->dim;
    TOG_TRY(tog_grid_counts(dim, desc->nel, nullptr, nullptr, nullptr));
    for (int d = 0; d < dim; ++d)
        if (!(desc->size[d] > 0)) return fail(TOG_ERR_ARG, "element sizes must be > 0");
    if (!(desc->E > 0) || !(desc->nu > -1.0 && desc->nu < 0.5)) return fail(TOG_ERR_ARG, "need E > 0 and -1 < nu < 0.5");
    if (!(desc->xmin >= 0 && desc->xmin < 1)) return fail(TOG_ERR_ARG, "xmin must be in [0, 1)");
    tog_handle* h = new tog_handle();
    h->dim = dim;
    for (int d = 0; d < 3; ++d) {
        h->nel[d] = d < dim ? desc->nel[d] : 1;
        h->nn[d] = d < dim ? desc->nel[d] + 1 : 1;
        h->size[d] = d < dim ? desc->size[d] : 1.0;
    }
    grid_counts(dim, desc->nel, &h->nnodes, &h->ncells);
    h->ndofs = h->nnodes * dim;
    if (h->ndofs >= (1LL << 31)) {
        delete h;
        return fail(TOG_ERR_ARG, "more than 2^31 dofs");
    }
    h->E = desc->E;
    h->nu = desc->nu;
    h->xmin = desc->xmin;
    h->p = desc->penalty;
    h->plane_stress = desc->plane_stress;
    // numbering
    h->node_dofs.resize(h->ndofs);
    node_dofs_first_touch(dim, desc->nel, h->node_dofs.data());
    h->ref2int.assign(h->ndofs, -1);
    for (long long i = 0; i < h->ndofs; ++i) h->ref2int[h->node_dofs[i]] = (int32_t)i;
    // element operator
    const int nd = (1 << dim) * dim;
    std::vector<double> Ke(nd * nd);
    element_stiffness(dim, h->size, h->E, h->nu, h->plane_stress, Ke.data());
    double tr = 0;
    for (int i = 0; i < nd; ++i) tr += Ke[i * nd + i];
    h->meandiag = tr * (double)h->ncells;   // sum of element traces (solvers_api.jl:526-527)
    double kd[3];
    try {
        if (dim == 3) {
            modal_operator(3, Ke.data(), &h->M3d.D[0][0], &h->M3d.O[0][0][0], kd);
            for (int m = 0; m < 8; ++m)
                for (int c = 0; c < 3; ++c) {
                    h->M3f.D[m][c] = (float)h->M3d.D[m][c];
                    for (int d = 0; d < 3; ++d) h->M3f.O[m][c][d] = (float)h->M3d.O[m][c][d];
                }
            for (int c = 0; c < 3; ++c) {
                h->M3d.kdinv[c] = 1.0 / kd[c];
                h->M3f.kdinv[c] = (float)(1.0 / kd[c]);
            }
        } else {
            modal_operator(2, Ke.data(), &h->M2d.D[0][0], &h->M2d.O[0][0][0], kd);
            for (int m = 0; m < 4; ++m)
                for (int c = 0; c < 2; ++c) {
                    h->M2f.D[m][c] = (float)h->M2d.D[m][c];
                    for (int d = 0; d < 2; ++d) h->M2f.O[m][c][d] = (float)h->M2d.O[m][c][d];
                }
            for (int c = 0; c < 2; ++c) {
                h->M2d.kdinv[c] = 1.0 / kd[c];
                h->M2f.kdinv[c] = (float)(1.0 / kd[c]);
            }
        }
    } catch (const std::exception& ex) {
        delete h;
        return fail(TOG_ERR_ARG, ex.what());
    }
    // device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return fail(TOG_ERR_CUDA, std::string("CUDA init: ") + cudaGetErrorString(e));
    }
    h->stream = h->own;
    if (const char* e = std::getenv("TOG_RU_DELTA")) h->ru_delta = std::min(0.9, std::max(1e-6, std::atof(e)));
    if (const char* e = std::getenv("TOG_UPD_BLOCKS_PER_SM")) h->upd_per_sm = std::min(32, std::max(1, std::atoi(e)));
    if (const char* e = std::getenv("TOG_PCG_UNROLL")) h->pcg_unroll = std::min(32, std::max(1, std::atoi(e)));
    if (dim == 3) {
        // z-chunk length: minimise (rounds of resident blocks) x (layers + prologue)
        h->nt[0] = (h->nel[0] + 31) / 32;
        h->nt[1] = (h->nel[1] + MV3_BY - 1) / MV3_BY;
        const long long txy = (long long)h->nt[0] * h->nt[1];
        int bps = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_march3, 32 * kM3Warps, 0) != cudaSuccess || bps < 1)
            bps = 1;
        h->march_grid = h->nsm * bps;
        {   // z bands: fewest (rounds of the warp grid) x (planes walked per band, halo included)
            const long long ncol = (long long)((h->nn[0] + 29) / 30) * h->nn[1];
            const long long gw = (long long)h->march_grid * kM3Warps;
            long long best = -1;
            for (int b = 1; b <= h->nn[2]; ++b) {
                const int lz = (h->nn[2] + b - 1) / b;
                const long long rounds = (ncol * b + gw - 1) / gw;
                const long long cost = rounds * (lz + 2);
                if (best < 0 || cost < best) {
                    best = cost;
                    h->march_nband = b;
                    h->march_lzb = lz;
                }
            }
        }
        int occ = 0;
        cudaError_t oe;
        // z chunks of the FP64 tile operator (k_mv3<double>: FP64 PCG, true residual, K x)
        cudaFuncSetAttribute(k_mv3<double, MV_PCG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(Mv3Smem<double>));
        oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mv3<double, MV_PCG>, 32 * MV3_BY,
                                                           sizeof(Mv3Smem<double>));
        if (oe != cudaSuccess || occ < 1) occ = 1;
        const long long slots = (long long)h->nsm * occ;
        int best = h->nel[2];
        double best_cost = 1e300;
        for (int lz = 2; lz <= h->nel[2]; ++lz) {
            const long long blocks = txy * ((h->nel[2] + lz - 1) / lz);
            const double cost = (double)((blocks + slots - 1) / slots) * (lz + 2);
            if (cost < best_cost) {
                best_cost = cost;
                best = lz;
            }
        }
        int lz = best;
        if (const char* e = std::getenv("TOG_MV3_LZ")) lz = std::max(1, std::atoi(e));
        h->LZ = lz;
        h->nt[2] = (h->nel[2] + lz - 1) / lz;
    }
    const long long N = h->ndofs, NN = h->nnodes, NC = h->ncells;
    // partial-sum buffer: enough for the largest grid of any reducing kernel
    const dim3 g3 = mv3_grid(h), g2 = mv2_grid(h);
    size_t maxb = (size_t)g3.x * g3.y * g3.z;
    maxb = std::max(maxb, (size_t)h->nt[0] * h->nt[1] * h->nt[2]);
    maxb = std::max(maxb, (size_t)((h->nnodes + kEwThreads - 1) / kEwThreads));
    maxb = std::max(maxb, (size_t)g2.x * g2.y);
    maxb = std::max(maxb, (size_t)h->nsm * 8);
    maxb = std::max(maxb, (size_t)h->march_grid);
    h->npartials = maxb * 4;
    int rc = TOG_OK;
    auto A = [&](int r) {
        if (rc == TOG_OK) rc = r;
    };
    A(dalloc(&h->d_int2ref, N));
    A(dalloc(&h->d_ref2int, N));
    A(dalloc(&h->d_fixmask, NN));

    A(dalloc(&h->d_vars, NC));
    A(dalloc(&h->d_e64, NC));
    A(dalloc(&h->d_e32, NC));
    A(dalloc(&h->d_dinv64, NN));
    A(dalloc(&h->d_dinv32, NN));
    {   // dof-sized vectors from one pool, base addresses staggered (pool_take)
        const size_t per64 = ((N * 8 + 13 * 1280 + 256 + 4095) / 4096) * 4096;
        const size_t per32 = ((N * 4 + 13 * 1280 + 256 + 4095) / 4096) * 4096;
        A(dalloc(&h->d_vecpool, 8 * per64 + 5 * per32));
        if (rc == TOG_OK) {
            char* cur = h->d_vecpool;
            int slot = 0;
            h->d_f = pool_take<double>(cur, N, slot++);
            h->d_u = pool_take<double>(cur, N, slot++);
            h->d_r64 = pool_take<double>(cur, N, slot++);
            h->d_p64[0] = pool_take<double>(cur, N, slot++);
            h->d_p64[1] = pool_take<double>(cur, N, slot++);
            h->d_q64 = pool_take<double>(cur, N, slot++);
            h->d_tmp = pool_take<double>(cur, N, slot++);
            h->d_tmp2 = pool_take<double>(cur, N, slot++);
            h->d_x32 = pool_take<float>(cur, N, slot++);
            h->d_r32 = pool_take<float>(cur, N, slot++);
            h->d_p32[0] = pool_take<float>(cur, N, slot++);
            h->d_p32[1] = pool_take<float>(cur, N, slot++);
            h->d_q32 = pool_take<float>(cur, N, slot++);
        }
    }
    for (int i = 0; i < 6; ++i) A(dalloc(&h->d_cell[i], NC));
    A(dalloc(&h->d_nodal, NN));
    A(dalloc(&h->d_st64, 1));
    A(dalloc(&h->d_st32, 1));
    A(dalloc(&h->d_oc, 1));
    A(dalloc(&h->d_partials, h->npartials));
    A(dalloc(&h->d_cnt, 8));
    A(dalloc(&h->d_scalar, 8));
    A(dalloc(&h->d_invW, NC));
    if (dim == 3)
        for (int c = 1; c < 8; ++c) {
            const long long cnt = 3 * std::max(1LL, side_count(c, h->nn, h->nt));
            A(dalloc(&h->d_side64[c], cnt));
        }
    if (rc == TOG_OK) {
        h->d_x = h->d_cell[0];
        h->d_xnew = h->d_cell[1];
        h->d_dc = h->d_cell[2];
        h->d_dv = h->d_cell[3];
        h->d_w = h->d_cell[4];
        h->d_grad = h->d_cell[5];
        h->d_B = h->d_tmp;   // OC scratch shares the dof staging buffer (ncells <= ndofs)
        cudaError_t ee = cudaSuccess;
        auto C = [&](cudaError_t x) {
            if (ee == cudaSuccess) ee = x;
        };
        C(cudaHostAlloc((void**)&h->h_st, 2 * sizeof(PcgState), cudaHostAllocDefault));   // FP32, FP64 segment states
        C(cudaHostAlloc((void**)&h->h_oc, sizeof(OcState), cudaHostAllocDefault));
        C(cudaHostAlloc((void**)&h->h_scalar, 8 * sizeof(double), cudaHostAllocDefault));
        C(cudaMemcpyAsync(h->d_int2ref, h->node_dofs.data(), N * sizeof(int), cudaMemcpyHostToDevice, h->own));
        C(cudaMemcpyAsync(h->d_ref2int, h->ref2int.data(), N * sizeof(int), cudaMemcpyHostToDevice, h->own));
        C(cudaMemsetAsync(h->d_fixmask, 0, NN, h->own));
        C(cudaMemsetAsync(h->d_f, 0, N * sizeof(double), h->own));
        C(cudaMemsetAsync(h->d_u, 0, N * sizeof(double), h->own));
        C(cudaMemsetAsync(h->d_st64, 0, sizeof(PcgState), h->own));
        C(cudaMemsetAsync(h->d_st32, 0, sizeof(PcgState), h->own));
        C(cudaMemsetAsync(h->d_oc, 0, sizeof(OcState), h->own));
        C(cudaMemsetAsync(h->d_cnt, 0, 8 * sizeof(unsigned), h->own));
        // vars = ones (solvers_api.jl:502)
        std::vector<double> ones(NC, 1.0);
        C(cudaMemcpyAsync(h->d_vars, ones.data(), NC * sizeof(double), cudaMemcpyHostToDevice, h->own));
        C(cudaStreamSynchronize(h->own));
        if (ee != cudaSuccess) rc = fail(TOG_ERR_CUDA, std::string("init: ") + cudaGetErrorString(ee));
    }
    if (rc != TOG_OK) {
        std::string msg = g_err;
        tog_destroy(h);
        g_err = msg;
        return rc;
    }
    h->vars_dirty = true;
    *out = h;
    return TOG_OK;
}

int tog_destroy(tog_handle* h) {
    if (!h) return TOG_OK;
    if (h->own) cudaStreamSynchronize(h->own);
    if (h->stream && h->stream != h->own) cudaStreamSynchronize(h->stream);
    if (h->g_pcg64) cudaGraphExecDestroy(h->g_pcg64);
    if (h->g_pcg32) cudaGraphExecDestroy(h->g_pcg32);
    if (h->g_pcg64e) cudaGraphExecDestroy(h->g_pcg64e);
    if (h->g_oc) cudaGraphExecDestroy(h->g_oc);
    if (h->g_mma) cudaGraphExecDestroy(h->g_mma);
    if (h->h_mma) cudaFreeHost(h->h_mma);
    void* ptrs[] = {h->d_int2ref, h->d_ref2int, h->d_fixmask, h->d_vecpool, h->d_vars,    h->d_e64,
                    h->d_e32,     h->d_dinv64,  h->d_dinv32,  h->d_nodal,   h->d_st64,    h->d_st32,
                    h->d_oc,      h->d_partials, h->d_cnt,    h->d_scalar,  h->d_invW,    h->d_soff,
                    h->d_sw,      h->d_vars_prev, h->d_uprev, h->d_du_last, h->d_nn_in, h->d_nn_out, h->d_nn_sc,
                    h->d_nn_part, h->d_nn_cnt, h->d_fpos, h->d_mma, h->d_mma_buf, h->d_mlg, h->d_fsave};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int i = 0; i < 6; ++i)
        if (h->d_cell[i]) cudaFree(h->d_cell[i]);
    for (int c = 0; c < 8; ++c) {
        if (h->d_side64[c]) cudaFree(h->d_side64[c]);
    }
    if (h->h_st) cudaFreeHost(h->h_st);
    if (h->h_oc) cudaFreeHost(h->h_oc);
    if (h->h_scalar) cudaFreeHost(h->h_scalar);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
    return TOG_OK;
}

int tog_set_stream(tog_handle* h, void* stream) {
    TOG_TRY(check_handle(h));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    h->stream = stream ? (cudaStream_t)stream : h->own;
    return TOG_OK;
}

int tog_set_fixed_dofs(tog_handle* h, int64_t n, const int32_t* dofs) {
    TOG_TRY(check_handle(h));
    if (n < 0 || (n > 0 && !dofs)) return fail(TOG_ERR_ARG, "bad fixed dof list");
    std::vector<uint8_t> mask(h->nnodes, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int32_t d = dofs[i];
        if (d < 0 || d >= h->ndofs) return fail(TOG_ERR_ARG, "fixed dof out of range");
        const int32_t k = h->ref2int[d];
        mask[k / h->dim] |= (uint8_t)(1u << (k % h->dim));
    }
    TOG_CUDA(cudaMemcpyAsync(h->d_fixmask, mask.data(), h->nnodes, cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    h->u_valid = false;
    return TOG_OK;
}

int tog_set_rhs(tog_handle* h, const double* f) {
    TOG_TRY(check_handle(h));
    if (!f) return fail(TOG_ERR_ARG, "null rhs");
    // masked copy: prescribed dofs carry no load (homogeneous Dirichlet, apply_zero!)
    std::vector<uint8_t> mask(h->nnodes);
    TOG_CUDA(cudaMemcpyAsync(mask.data(), h->d_fixmask, h->nnodes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<double> fi(h->ndofs);
    double s = 0;
    for (long long i = 0; i < h->ndofs; ++i) {
        const bool fixed = (mask[i / h->dim] >> (i % h->dim)) & 1u;
        const double v = fixed ? 0.0 : f[h->node_dofs[i]];
        if (!std::isfinite(v)) return fail(TOG_ERR_ARG, "rhs has non-finite entries");
        fi[i] = v;
        s += v * v;
    }
    h->fnorm2 = s;
    TOG_CUDA(cudaMemcpyAsync(h->d_f, fi.data(), h->ndofs * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_set_convergence(tog_handle* h, int32_t criteria) {
    TOG_TRY(check_handle(h));
    if (criteria != TOG_CONV_DEFAULT && criteria != TOG_CONV_ENERGY) return fail(TOG_ERR_ARG, "unknown criteria");
    h->conv = criteria;
    return TOG_OK;
}

int tog_set_penalty(tog_handle* h, double p) {
    TOG_TRY(check_handle(h));
    if (!(p >= 0) || !std::isfinite(p)) return fail(TOG_ERR_ARG, "penalty must be finite and >= 0");
    h->p = p;
    h->vars_dirty = true;
    return TOG_OK;
}

int tog_set_vars(tog_handle* h, const double* x) {
    TOG_TRY(check_handle(h));
    if (!x) return fail(TOG_ERR_ARG, "null vars");
    for (long long e = 0; e < h->ncells; ++e)
        if (!std::isfinite(x[e])) return fail(TOG_ERR_ARG, "vars has non-finite entries");
    TOG_CUDA(cudaMemcpyAsync(h->d_vars, x, h->ncells * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->vars_dirty = true;
    return TOG_OK;
}

int tog_matvec(tog_handle* h, const double* x, double* y) {
    TOG_TRY(check_handle(h));
    if (!x || !y) return fail(TOG_ERR_ARG, "null vector");
    TOG_TRY(refresh_scales(h));
    TOG_TRY(upload_dofs(h, x, h->d_p64[0]));
    launch_matvec<double, MV_PLAIN>(h, h->stream, h->d_p64[0], h->d_r64, nullptr);
    TOG_CUDA(cudaGetLastError());
    return download_dofs(h, h->d_r64, y);
}

// One fused PCG operator launch on caller vectors (the kernel every PCG iteration
// runs first): p = D^-1 r + beta p_old, q = K(rho) p with the prescribed rows set
// to meandiag p (as the PCG update uses it), p.q.
int tog_pcg_operator(tog_handle* h, int32_t precision, double beta, const double* r, const double* p_old, double* p,
                     double* q, double* pq) {
    TOG_TRY(check_handle(h));
    if (!r || !p_old || !p || !q) return fail(TOG_ERR_ARG, "null vector");
    if (precision != TOG_FP64 && precision != TOG_FP32_IR) return fail(TOG_ERR_ARG, "bad precision");
    if (!std::isfinite(beta)) return fail(TOG_ERR_ARG, "beta must be finite");
    TOG_TRY(refresh_scales(h));
    const bool f32 = precision == TOG_FP32_IR;
    const long long nd = h->ndofs;
    const int nb = h->ew_blocks(nd);
    PcgState* d_st = f32 ? h->d_st32 : h->d_st64;
    if (f32) {
        TOG_TRY(upload_dofs(h, r, h->d_tmp));
        k_cast_f32<<<nb, kEwThreads, 0, h->stream>>>(h->d_tmp, h->d_r32, nd);
        TOG_TRY(upload_dofs(h, p_old, h->d_tmp));
        k_cast_f32<<<nb, kEwThreads, 0, h->stream>>>(h->d_tmp, h->d_p32[1], nd);
        TOG_LAUNCHED(2);
    } else {
        TOG_TRY(upload_dofs(h, r, h->d_r64));
        TOG_TRY(upload_dofs(h, p_old, h->d_p64[1]));
    }
    // iteration 0 (direction into P0, previous direction from P1), r.z = 1
    PcgState* hs = h->h_st;
    std::memset(hs, 0, sizeof(PcgState));
    hs->rz = 1.0;
    hs->beta = beta;
    hs->maxit = 1 << 30;
    TOG_CUDA(cudaMemcpyAsync(d_st, hs, sizeof(PcgState), cudaMemcpyHostToDevice, h->stream));
    if (f32) {
        launch_matvec<float, MV_PCG>(h, h->stream, nullptr, nullptr, nullptr);
        k_pcg_operator_out<float><<<h->ew_blocks(h->nnodes), kEwThreads, 0, h->stream>>>(
            h->d_p32[0], h->d_q32, h->d_fixmask, h->meandiag, h->nnodes, h->dim, h->d_tmp, h->d_r64);
    } else {
        launch_matvec<double, MV_PCG>(h, h->stream, nullptr, nullptr, nullptr);
        if (h->dim == 3) {   // the tile operator leaves tile-boundary partials for the PCG update to gather
            Mv3Args<double> A = mv3_args<double>(h);
            k_side_gather3<double><<<h->ew_blocks(h->nnodes), kEwThreads, 0, h->stream>>>(A);
            TOG_LAUNCHED(1);
        }
        k_pcg_operator_out<double><<<h->ew_blocks(h->nnodes), kEwThreads, 0, h->stream>>>(
            h->d_p64[0], h->d_q64, h->d_fixmask, h->meandiag, h->nnodes, h->dim, h->d_tmp, h->d_r64);
    }
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    TOG_TRY(sync_state(h, d_st));
    if (pq) *pq = h->h_st->pq;
    TOG_TRY(download_dofs(h, h->d_tmp, p));
    return download_dofs(h, h->d_r64, q);
}

int tog_solve(tog_handle* h, int32_t precision, double rtol, double abstol, int32_t maxiter, int32_t warm_start,
              tog_solve_stats* stats) {
    TOG_TRY(check_handle(h));
    if (!(rtol >= 0) || !(abstol >= 0) || maxiter < 0) return fail(TOG_ERR_ARG, "bad tolerance or maxiter");
    return do_solve(h, precision, rtol, abstol, maxiter, warm_start, stats);
}

int tog_get_u(tog_handle* h, double* u) {
    TOG_TRY(check_handle(h));
    if (!u) return fail(TOG_ERR_ARG, "null output");
    return download_dofs(h, h->d_u, u);
}

int tog_set_u(tog_handle* h, const double* u) {
    TOG_TRY(check_handle(h));
    if (!u) return fail(TOG_ERR_ARG, "null input");
    TOG_TRY(upload_dofs(h, u, h->d_u));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    h->u_valid = true;
    return TOG_OK;
}

// rhs column scatter: f[idx[k]] = val[k] (f zeroed before; prescribed dofs already dropped)
__global__ void k_scatter_pairs(double* __restrict__ f, const long long* __restrict__ idx,
                                const double* __restrict__ val, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) f[idx[k]] = val[k];
}
// out = sum_i w_i g_i over the per-column cell gradients (column-major ncells x ncol)
__global__ void __launch_bounds__(256) k_weighted_cols(const double* __restrict__ g, const double* __restrict__ w,
                                                       int ncol, long long ncells, double* __restrict__ out) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncells;
         e += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int i = 0; i < ncol; ++i) acc = fma(w[i], g[(size_t)i * ncells + e], acc);
        out[e] = acc;
    }
}

int tog_multiload_compliance(tog_handle* h, int32_t ncol, const int64_t* colptr, const int32_t* rowval,
                             const double* nzval, int32_t precision, double rtol, double abstol, int32_t maxiter,
                             double* c, tog_solve_stats* stats) {
    TOG_TRY(check_handle(h));
    if (ncol <= 0 || !colptr || !c || (colptr[ncol] > 0 && (!rowval || !nzval)))
        return fail(TOG_ERR_ARG, "need ncol > 0, colptr[ncol + 1], rowval, nzval and c[ncol]");
    if (colptr[0] != 0) return fail(TOG_ERR_ARG, "colptr[0] must be 0");
    for (int i = 0; i < ncol; ++i)
        if (colptr[i + 1] < colptr[i]) return fail(TOG_ERR_ARG, "colptr must be non-decreasing");
    for (long long k = 0; k < colptr[ncol]; ++k) {
        if (rowval[k] < 0 || rowval[k] >= h->ndofs) return fail(TOG_ERR_ARG, "rhs row out of range");
        if (!std::isfinite(nzval[k])) return fail(TOG_ERR_ARG, "rhs has non-finite entries");
    }
    std::vector<uint8_t> mask(h->nnodes);
    TOG_CUDA(cudaMemcpyAsync(mask.data(), h->d_fixmask, h->nnodes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    if (h->mlg_cols < ncol) {
        if (h->d_mlg) cudaFree(h->d_mlg);
        h->d_mlg = nullptr;
        h->mlg_cols = 0;
        TOG_TRY(dalloc(&h->d_mlg, (size_t)ncol * h->ncells));
        h->mlg_cols = ncol;
    }
    if (!h->d_fsave) TOG_TRY(dalloc(&h->d_fsave, h->ndofs));
    const size_t fbytes = h->ndofs * sizeof(double);
    TOG_CUDA(cudaMemcpyAsync(h->d_fsave, h->d_f, fbytes, cudaMemcpyDeviceToDevice, h->stream));
    const double fnorm_saved = h->fnorm2;
    long long maxnz = 1;
    for (int i = 0; i < ncol; ++i) maxnz = std::max<long long>(maxnz, colptr[i + 1] - colptr[i]);
    long long* d_idx = nullptr;
    double* d_val = nullptr;
    TOG_TRY(dalloc(&d_idx, maxnz));
    if (dalloc(&d_val, maxnz) != TOG_OK) {
        cudaFree(d_idx);
        return TOG_ERR_OOM;
    }
    int rc = TOG_OK;
    long long its = 0;
    tog_solve_stats ss{};
    std::vector<long long> idx;
    std::vector<double> val;
    for (int i = 0; i < ncol && (rc == TOG_OK || rc == TOG_NOT_CONVERGED); ++i) {
        // column i with its prescribed dofs zeroed (apply_zero!), summed per internal dof
        idx.clear();
        val.clear();
        std::vector<std::pair<long long, double>> ent;
        for (long long k = colptr[i]; k < colptr[i + 1]; ++k) {
            const long long ii = h->ref2int[rowval[k]];
            if ((mask[ii / h->dim] >> (ii % h->dim)) & 1u) continue;
            ent.emplace_back(ii, nzval[k]);
        }
        std::sort(ent.begin(), ent.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        double s2 = 0.0;
        for (size_t k = 0; k < ent.size(); ++k) {
            if (!idx.empty() && idx.back() == ent[k].first)
                val.back() += ent[k].second;
            else {
                idx.push_back(ent[k].first);
                val.push_back(ent[k].second);
            }
        }
        for (double v : val) s2 += v * v;
        h->fnorm2 = s2;
        auto cu = [&](cudaError_t e) {
            if (e != cudaSuccess && rc == TOG_OK) rc = fail(TOG_ERR_CUDA, cudaGetErrorString(e));
        };
        cu(cudaMemsetAsync(h->d_f, 0, fbytes, h->stream));
        if (!idx.empty()) {
            cu(cudaMemcpyAsync(d_idx, idx.data(), idx.size() * sizeof(long long), cudaMemcpyHostToDevice, h->stream));
            cu(cudaMemcpyAsync(d_val, val.data(), val.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            k_scatter_pairs<<<std::min<int>(1024, ((int)idx.size() + 255) / 256), 256, 0, h->stream>>>(
                h->d_f, d_idx, d_val, (int)idx.size());
            TOG_LAUNCHED(1);
            cu(cudaGetLastError());
            cu(cudaStreamSynchronize(h->stream));   // the host pairs are reused by the next column
        }
        if (rc != TOG_OK) break;
        const int r = do_solve(h, precision, rtol, abstol, maxiter, 0, &ss);   // each column from zero
        its += ss.iterations;
        if (r != TOG_OK && r != TOG_NOT_CONVERGED) {
            rc = r;
            break;
        }
        if (r == TOG_NOT_CONVERGED) rc = r;
        const int rc2 = compliance_dev(h, h->d_mlg + (size_t)i * h->ncells);
        if (rc2 != TOG_OK) {
            rc = rc2;
            break;
        }
        cu(cudaMemcpyAsync(h->h_scalar, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        cu(cudaStreamSynchronize(h->stream));
        c[i] = h->h_scalar[0];
    }
    cudaStreamSynchronize(h->stream);
    cudaFree(d_idx);
    cudaFree(d_val);
    // the handle's own rhs again (the displacement stays that of the last column)
    TOG_CUDA(cudaMemcpyAsync(h->d_f, h->d_fsave, fbytes, cudaMemcpyDeviceToDevice, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    h->fnorm2 = fnorm_saved;
    if (stats) {
        *stats = ss;
        stats->iterations = (int32_t)std::min<long long>(its, INT32_MAX);
    }
    return rc;
}

int tog_multiload_gradient(tog_handle* h, int32_t ncol, const double* w, double* out) {
    TOG_TRY(check_handle(h));
    if (!w || !out || ncol <= 0) return fail(TOG_ERR_ARG, "need ncol > 0, w[ncol] and out[ncells]");
    if (!h->d_mlg || ncol > h->mlg_cols) return fail(TOG_ERR_STATE, "no multi-load gradients: call tog_multiload_compliance first");
    double* d_wc = nullptr;
    TOG_TRY(dalloc(&d_wc, ncol));
    TOG_CUDA(cudaMemcpyAsync(d_wc, w, ncol * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    k_weighted_cols<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_mlg, d_wc, ncol, h->ncells, h->d_grad);
    TOG_LAUNCHED(1);
    const cudaError_t e = cudaGetLastError();
    TOG_CUDA(cudaMemcpyAsync(out, h->d_grad, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    cudaFree(d_wc);
    TOG_CUDA(e);
    return TOG_OK;
}

int tog_compliance(tog_handle* h, double* c, double* grad) {
    TOG_TRY(check_handle(h));
    if (!h->u_valid) return fail(TOG_ERR_STATE, "no displacement: call tog_solve first");
    TOG_TRY(compliance_dev(h, h->d_grad));
    if (grad)
        TOG_CUDA(cudaMemcpyAsync(grad, h->d_grad, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->h_scalar, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    if (c) *c = h->h_scalar[0];
    return TOG_OK;
}

int tog_filter_setup(tog_handle* h, double rmin) {
    TOG_TRY(check_handle(h));
    if (!(rmin > 0) || !std::isfinite(rmin)) return fail(TOG_ERR_ARG, "rmin must be > 0");
    std::vector<int> off;
    std::vector<double> w;
    const int S = filter_stencil(h->dim, h->size, rmin, off, w);
    if (S == 0)
        return fail(TOG_ERR_ARG,
                    "DensityFilterFun: no neighbouring nodes were found within the filter radius rmin for any "
                    "element; rmin is likely smaller than the element size");
    if (h->d_soff) cudaFree(h->d_soff);
    if (h->d_sw) cudaFree(h->d_sw);
    h->d_soff = nullptr;
    h->d_sw = nullptr;
    TOG_TRY(dalloc(&h->d_soff, off.size()));
    TOG_TRY(dalloc(&h->d_sw, w.size()));
    TOG_CUDA(cudaMemcpyAsync(h->d_soff, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_sw, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->S = S;
    {   // the stencil's node-offset box decides between the fused and the two-pass kernels
        FiltBox B{};
        for (int d = 0; d < 3; ++d) {
            B.lo[d] = 1 << 30;
            B.hi[d] = -(1 << 30);
        }
        for (int k = 0; k < S; ++k)
            for (int d = 0; d < 3; ++d) {
                B.lo[d] = std::min(B.lo[d], off[3 * k + d]);
                B.hi[d] = std::max(B.hi[d], off[3 * k + d]);
            }
        h->fbox = B;
        h->filt_smem[0] = filt_fwd_smem(B, S, h->dim);
        h->filt_smem[1] = filt_bwd_smem(B, S, h->dim);
        h->filt_fused = std::max(h->filt_smem[0], h->filt_smem[1]) <= kFiltMaxSmem;
        if (h->filt_fused) {
            if (h->dim == 3) {
                TOG_CUDA(cudaFuncSetAttribute(k_filt_fwd<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)h->filt_smem[0]));
                TOG_CUDA(cudaFuncSetAttribute(k_filt_bwd<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)h->filt_smem[1]));
                // z bands: about two blocks per SM, at least 8 cell planes each
                const long long tiles = (long long)((h->nel[0] + kFiltTX - 1) / kFiltTX) *
                                        ((h->nel[1] + kFiltTY - 1) / kFiltTY);
                long long nb = std::max(1LL, (2LL * h->nsm + tiles - 1) / tiles);
                nb = std::min<long long>(nb, std::max(1, h->nel[2] / 8));
                h->filt_lz = (int)((h->nel[2] + nb - 1) / nb);
            } else {
                TOG_CUDA(cudaFuncSetAttribute(k_filt_fwd<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)h->filt_smem[0]));
                TOG_CUDA(cudaFuncSetAttribute(k_filt_bwd<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)h->filt_smem[1]));
                h->filt_lz = 1;
            }
        }
    }
    if (h->dim == 3)
        k_filt_invW<3><<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_soff, h->d_sw, S, h->d_invW,
                                                                              h->dims());
    else
        k_filt_invW<2><<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_soff, h->d_sw, S, h->d_invW,
                                                                              h->dims());
    TOG_LAUNCHED(1);
    TOG_CUDA(cudaGetLastError());
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    h->filter_ready = true;
    h->rmin = rmin;
    return TOG_OK;
}

int tog_filter_apply(tog_handle* h, int32_t op, const double* in, double* out) {
    TOG_TRY(check_handle(h));
    if (!h->filter_ready) return fail(TOG_ERR_STATE, "tog_filter_setup has not been called");
    if (!in || !out || (op != TOG_FILTER_J && op != TOG_FILTER_JT)) return fail(TOG_ERR_ARG, "bad filter arguments");
    const size_t bytes = h->ncells * sizeof(double);
    TOG_CUDA(cudaMemcpyAsync(h->d_xnew, in, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_TRY(filter_dev(h, op, h->d_xnew, h->d_grad));
    TOG_CUDA(cudaMemcpyAsync(out, h->d_grad, bytes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_projection(tog_handle* h, int32_t kind, double beta, const double* x, double* y, double* dydx) {
    TOG_TRY(check_handle(h));
    if (!x || !y || !dydx) return fail(TOG_ERR_ARG, "null array");
    if (kind != TOG_PROJ_HEAVISIDE && kind != TOG_PROJ_SIGMOID) return fail(TOG_ERR_ARG, "unknown projection");
    if (!std::isfinite(beta) || beta < 0) return fail(TOG_ERR_ARG, "projection steepness must be finite and >= 0");
    const size_t bytes = h->ncells * sizeof(double);
    TOG_CUDA(cudaMemcpyAsync(h->d_xnew, x, bytes, cudaMemcpyHostToDevice, h->stream));
    k_projection<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(kind, beta, h->d_xnew, h->d_grad, h->d_dc,
                                                                       h->ncells);
    TOG_CUDA(cudaGetLastError());
    TOG_CUDA(cudaMemcpyAsync(y, h->d_grad, bytes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaMemcpyAsync(dydx, h->d_dc, bytes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_set_fixed_elements(tog_handle* h, const uint8_t* state) {
    TOG_TRY(check_handle(h));
    if (!state) {   // every cell free
        if (h->d_fpos) {
            TOG_CUDA(cudaStreamSynchronize(h->stream));
            cudaFree(h->d_fpos);
            h->d_fpos = nullptr;
        }
        h->nfree = h->ncells;
    } else {
        if (h->ncells >= (1LL << 31)) return fail(TOG_ERR_ARG, "the active-element mask needs fewer than 2^31 cells");
        std::vector<int> pos(h->ncells);
        long long nf = 0;
        for (long long e = 0; e < h->ncells; ++e) {
            if (state[e] > TOG_ELEM_WHITE)
                return fail(TOG_ERR_ARG, "element state must be 0 (free), 1 (black) or 2 (white), cell " +
                                             std::to_string(e) + " has " + std::to_string((int)state[e]));
            pos[e] = state[e] == TOG_ELEM_FREE ? (int)nf++ : (state[e] == TOG_ELEM_BLACK ? -1 : -2);
        }
        if (!h->d_fpos) TOG_TRY(dalloc(&h->d_fpos, h->ncells));
        TOG_CUDA(cudaMemcpyAsync(h->d_fpos, pos.data(), h->ncells * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        TOG_CUDA(cudaStreamSynchronize(h->stream));
        h->nfree = nf;
    }
    // the OC graph holds the mask pointer: capture it again on the next update
    if (h->g_oc || h->g_mma) {
        TOG_CUDA(cudaStreamSynchronize(h->stream));
        if (h->g_oc) cudaGraphExecDestroy(h->g_oc);
        if (h->g_mma) cudaGraphExecDestroy(h->g_mma);
        h->g_oc = nullptr;
        h->g_mma = nullptr;
    }
    if (h->d_fpos && h->simp_ready) {   // an active loop's design follows the new mask at once
        k_fixed_pin<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_x, h->d_fpos, h->ncells);
        TOG_LAUNCHED(1);
        TOG_CUDA(cudaGetLastError());
        TOG_CUDA(cudaStreamSynchronize(h->stream));
    }
    return TOG_OK;
}

int tog_free_variable_count(tog_handle* h, int64_t* nfree) {
    TOG_TRY(check_handle(h));
    if (!nfree) return fail(TOG_ERR_ARG, "null output");
    *nfree = h->d_fpos ? h->nfree : h->ncells;
    return TOG_OK;
}

int tog_fixed_element_project(tog_handle* h, const double* x_free, int64_t nfree, double* rho) {
    TOG_TRY(check_handle(h));
    const long long nf = h->d_fpos ? h->nfree : h->ncells;
    if (nfree != nf)
        return fail(TOG_ERR_ARG, "x_free length (" + std::to_string((long long)nfree) +
                                     ") must match number of free elements (" + std::to_string(nf) + ")");
    if (!rho || (nf > 0 && !x_free)) return fail(TOG_ERR_ARG, "null array");
    if (nf > 0)
        TOG_CUDA(cudaMemcpyAsync(h->d_xnew, x_free, nf * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (h->d_fpos) {
        k_fixed_project<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_xnew, h->d_fpos, h->d_grad,
                                                                              h->ncells);
        TOG_LAUNCHED(1);
        TOG_CUDA(cudaGetLastError());
        TOG_CUDA(cudaMemcpyAsync(rho, h->d_grad, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    } else {
        TOG_CUDA(cudaMemcpyAsync(rho, h->d_xnew, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_fixed_element_pullback(tog_handle* h, const double* drho, double* dx_free) {
    TOG_TRY(check_handle(h));
    const long long nf = h->d_fpos ? h->nfree : h->ncells;
    if (!drho || (nf > 0 && !dx_free)) return fail(TOG_ERR_ARG, "null array");
    TOG_CUDA(cudaMemcpyAsync(h->d_xnew, drho, h->ncells * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (h->d_fpos) {
        k_fixed_pullback<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_xnew, h->d_fpos, h->d_grad,
                                                                               h->ncells);
        TOG_LAUNCHED(1);
        TOG_CUDA(cudaGetLastError());
        if (nf > 0)
            TOG_CUDA(cudaMemcpyAsync(dx_free, h->d_grad, nf * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    } else {
        TOG_CUDA(cudaMemcpyAsync(dx_free, h->d_xnew, nf * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_oc_update(tog_handle* h, const double* x, const double* dc, const double* dv, const double* vol_weights,
                  double volfrac, double move, double* x_new, double* change, double* lambda) {
    TOG_TRY(check_handle(h));
    if (!x || !dc || !dv || !vol_weights || !x_new) return fail(TOG_ERR_ARG, "null array");
    if (!(move > 0) || !(volfrac > 0 && volfrac <= 1)) return fail(TOG_ERR_ARG, "need move > 0 and 0 < volfrac <= 1");
    if (h->simp_ready) return fail(TOG_ERR_STATE, "tog_oc_update shares buffers with an active tog_simp loop");
    const size_t bytes = h->ncells * sizeof(double);
    TOG_CUDA(cudaMemcpyAsync(h->d_x, x, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_dc, dc, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_dv, dv, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_w, vol_weights, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_TRY(oc_dev(h, volfrac, move));
    TOG_CUDA(cudaMemcpyAsync(x_new, h->d_xnew, bytes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    if (change) *change = h->h_oc->change;
    if (lambda) *lambda = h->h_oc->lmid;
    return TOG_OK;
}

int tog_mma_update(tog_handle* h, const double* x, const double* df0, double g, const double* dg, double move,
                   double* x_new, double* change, double* lambda) {
    TOG_TRY(check_handle(h));
    if (!x || !df0 || !dg || !x_new) return fail(TOG_ERR_ARG, "null array");
    if (!(move > 0 && move <= 1) || !std::isfinite(g)) return fail(TOG_ERR_ARG, "need 0 < move <= 1 and a finite g");
    if (h->simp_ready) return fail(TOG_ERR_STATE, "tog_mma_update shares buffers with an active tog_simp loop");
    const size_t bytes = h->ncells * sizeof(double);
    TOG_CUDA(cudaMemcpyAsync(h->d_x, x, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_dc, df0, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_dv, dg, bytes, cudaMemcpyHostToDevice, h->stream));
    TOG_TRY(mma_dev(h, false, g, 0.0, move));
    TOG_CUDA(cudaMemcpyAsync(x_new, h->d_xnew, bytes, cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    if (change) *change = h->h_mma->change;
    if (lambda) *lambda = h->h_mma->lam;
    return TOG_OK;
}

int tog_mma_reset(tog_handle* h) {
    TOG_TRY(check_handle(h));
    h->mma_k = 0;
    return TOG_OK;
}

int tog_simp_set_optimizer(tog_handle* h, int32_t optimizer, double move) {
    TOG_TRY(check_handle(h));
    if (optimizer != TOG_OPT_OC && optimizer != TOG_OPT_MMA) return fail(TOG_ERR_ARG, "unknown optimizer");
    if (optimizer == TOG_OPT_MMA) {
        if (!(move <= 1)) return fail(TOG_ERR_ARG, "need move <= 1 (<= 0: the default 0.5)");
        h->mma_move = move > 0 ? move : 0.5;
    }
    h->simp_opt = optimizer;
    h->mma_k = 0;
    return TOG_OK;
}

int tog_simp_init(tog_handle* h, int32_t filter_kind, double rmin, double volfrac, double move, const double* x0) {
    TOG_TRY(check_handle(h));
    if (!x0) return fail(TOG_ERR_ARG, "null x0");
    if (filter_kind < TOG_FILTER_NONE || filter_kind > TOG_FILTER_SENS) return fail(TOG_ERR_ARG, "bad filter kind");
    if (!(move > 0) || !(volfrac > 0 && volfrac <= 1)) return fail(TOG_ERR_ARG, "need move > 0 and 0 < volfrac <= 1");
    if (filter_kind != TOG_FILTER_NONE) TOG_TRY(tog_filter_setup(h, rmin));
    h->simp_filter = filter_kind;
    h->volfrac = volfrac;
    h->move = move;
    const size_t bytes = h->ncells * sizeof(double);
    TOG_CUDA(cudaMemcpyAsync(h->d_x, x0, bytes, cudaMemcpyHostToDevice, h->stream));
    if (h->d_fpos) {   // fixed cells start (and stay) at their densities
        k_fixed_pin<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_x, h->d_fpos, h->ncells);
        TOG_LAUNCHED(1);
        TOG_CUDA(cudaGetLastError());
    }
    // dv = d(volume fraction)/dx; for the density filter dv = J' (1/n) (volume.jl:59-67 + filter rrule),
    // which is also the weight of x in the filtered volume used by the OC bisection.
    std::vector<double> inv(h->ncells, 1.0 / (double)h->ncells);
    TOG_CUDA(cudaMemcpyAsync(h->d_xnew, inv.data(), bytes, cudaMemcpyHostToDevice, h->stream));
    if (filter_kind == TOG_FILTER_DENSITY) {
        TOG_TRY(filter_dev(h, TOG_FILTER_JT, h->d_xnew, h->d_dv));
    } else {
        TOG_CUDA(cudaMemcpyAsync(h->d_dv, h->d_xnew, bytes, cudaMemcpyDeviceToDevice, h->stream));
    }
    TOG_CUDA(cudaMemcpyAsync(h->d_w, h->d_dv, bytes, cudaMemcpyDeviceToDevice, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    h->simp_ready = true;
    h->u_valid = false;
    h->mma_k = 0;
    return TOG_OK;
}

int tog_simp_step(tog_handle* h, int32_t precision, double rtol, int32_t maxiter, int32_t warm_start,
                  tog_iter_stats* stats) {
    TOG_TRY(check_handle(h));
    if (!h->simp_ready) return fail(TOG_ERR_STATE, "tog_simp_init has not been called");
    const size_t bytes = h->ncells * sizeof(double);
    // physical densities
    if (h->simp_filter == TOG_FILTER_DENSITY)
        TOG_TRY(filter_dev(h, TOG_FILTER_J, h->d_x, h->d_vars));
    else
        TOG_CUDA(cudaMemcpyAsync(h->d_vars, h->d_x, bytes, cudaMemcpyDeviceToDevice, h->stream));
    h->vars_dirty = true;
    // learned warm start / recording: need the previous iteration's densities and solution
    const bool prev_ok = h->d_vars_prev && h->have_prev && h->u_valid && h->dim == 3;
    const bool learned = warm_start == TOG_WARM_LEARNED && h->net && prev_ok;
    const bool extrap = (warm_start == TOG_WARM_LEARNED || warm_start == TOG_WARM_EXTRAPOLATE) && prev_ok;
    const bool record = h->rec_in && prev_ok;
    if (!record) h->rec_in = nullptr;
    const bool keep = prev_ok;   // u_prev is kept for the next iteration's last change
    if (learned || extrap || record || keep) TOG_TRY(nn_before_solve(h, learned, extrap));
    tog_solve_stats ss{};
    int rc = do_solve(h, precision, rtol, 0.0, maxiter, warm_start != 0, &ss);
    if (rc != TOG_OK && rc != TOG_NOT_CONVERGED) return rc;
    if (learned) TOG_TRY(nn_status(h->net, h->stream));
    if (record) {
        k_nn_target<<<h->ew_blocks(h->ndofs), kEwThreads, 0, h->stream>>>(h->d_u, h->d_uprev, h->d_nn_sc, h->rec_tgt,
                                                                         h->ndofs);
        h->rec_written = 1;
    }
    if (keep) {   // last change, for the next iteration's extrapolated / learned start
        k_sub<<<h->ew_blocks(h->ndofs), kEwThreads, 0, h->stream>>>(h->d_u, h->d_uprev, h->d_du_last, h->ndofs);
        h->have_du = true;
    }
    h->rec_in = nullptr;
    h->rec_tgt = nullptr;
    if (h->d_vars_prev) {
        TOG_CUDA(cudaMemcpyAsync(h->d_vars_prev, h->d_vars, bytes, cudaMemcpyDeviceToDevice, h->stream));
        h->have_prev = true;
    }
    TOG_TRY(compliance_dev(h, h->d_grad));
    if (h->simp_filter == TOG_FILTER_DENSITY)
        TOG_TRY(filter_dev(h, TOG_FILTER_JT, h->d_grad, h->d_dc));
    else if (h->simp_filter == TOG_FILTER_SENS)
        TOG_TRY(filter_dev(h, TOG_FILTER_J, h->d_grad, h->d_dc));
    else
        TOG_CUDA(cudaMemcpyAsync(h->d_dc, h->d_grad, bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (h->simp_opt == TOG_OPT_MMA)
        TOG_TRY(mma_dev(h, true, 0.0, h->volfrac, h->mma_move));
    else
        TOG_TRY(oc_dev(h, h->volfrac, h->move));
    TOG_CUDA(cudaMemcpyAsync(h->h_scalar, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    TOG_CUDA(cudaMemcpyAsync(h->d_x, h->d_xnew, bytes, cudaMemcpyDeviceToDevice, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    if (stats) {
        const bool mma = h->simp_opt == TOG_OPT_MMA;
        stats->compliance = h->h_scalar[0];
        stats->volume = mma ? h->h_mma->vol : h->h_oc->vol;
        stats->change = mma ? h->h_mma->change : h->h_oc->change;
        stats->lambda = mma ? h->h_mma->lam : h->h_oc->lmid;
        stats->cg_iterations = ss.iterations;
        stats->outer_iterations = ss.outer_iterations;
        stats->oc_steps = mma ? h->h_mma->steps : h->h_oc->steps;
        stats->status = ss.status;
        stats->rel_residual = ss.rel_residual;
    }
    return rc;
}

int tog_set_warm_start_net(tog_handle* h, tog_nn* nn) {
    TOG_TRY(check_handle(h));
    if (nn) {
        if (h->dim != 3) return fail(TOG_ERR_ARG, "the learned warm start is for 3D grids");
        const int nodes[3] = {h->nn[0], h->nn[1], h->nn[2]};
        if (!nn_matches(nn, nodes, 1))
            return fail(TOG_ERR_ARG, "network created for another node grid (or a batch other than 1)");
        TOG_TRY(nn_buffers(h));
    }
    h->net = nn;
    return TOG_OK;
}

int tog_keep_previous_state(tog_handle* h) {
    TOG_TRY(check_handle(h));
    if (h->dim != 3) return fail(TOG_ERR_ARG, "previous-state starts are for 3D grids");
    return nn_buffers(h);
}

int tog_record_next_step(tog_handle* h, float* input_dev, float* target_dev) {
    TOG_TRY(check_handle(h));
    if (!input_dev || !target_dev) return fail(TOG_ERR_ARG, "null recording buffer");
    if (h->dim != 3) return fail(TOG_ERR_ARG, "recording is for 3D grids");
    TOG_TRY(nn_buffers(h));
    h->rec_in = input_dev;
    h->rec_tgt = target_dev;
    h->rec_written = 0;
    return TOG_OK;
}

int tog_record_status(tog_handle* h, int32_t* written) {
    TOG_TRY(check_handle(h));
    if (!written) return fail(TOG_ERR_ARG, "null output");
    *written = h->rec_written;
    return TOG_OK;
}

int tog_get_design(tog_handle* h, double* x) {
    TOG_TRY(check_handle(h));
    if (!x) return fail(TOG_ERR_ARG, "null output");
    TOG_CUDA(cudaMemcpyAsync(x, h->d_x, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_set_design(tog_handle* h, const double* x) {
    TOG_TRY(check_handle(h));
    if (!x) return fail(TOG_ERR_ARG, "null input");
    TOG_CUDA(cudaMemcpyAsync(h->d_x, x, h->ncells * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (h->d_fpos) {
        k_fixed_pin<<<h->ew_blocks(h->ncells), kEwThreads, 0, h->stream>>>(h->d_x, h->d_fpos, h->ncells);
        TOG_LAUNCHED(1);
        TOG_CUDA(cudaGetLastError());
    }
    return TOG_OK;
}

int tog_get_physical(tog_handle* h, double* xf) {
    TOG_TRY(check_handle(h));
    if (!xf) return fail(TOG_ERR_ARG, "null output");
    TOG_CUDA(cudaMemcpyAsync(xf, h->d_vars, h->ncells * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TOG_CUDA(cudaStreamSynchronize(h->stream));
    return TOG_OK;
}

int tog_bench_kernel(tog_handle* h, int32_t kernel, int32_t precision, int32_t nlaunch) {
    TOG_TRY(check_handle(h));
    if (nlaunch < 0 || kernel < 0 || kernel > 1) return fail(TOG_ERR_ARG, "bad kernel id or nlaunch");
    TOG_TRY(refresh_scales(h));
    if (h->fnorm2 <= 0) return fail(TOG_ERR_STATE, "set a non-zero rhs first");
    // fresh PCG state from r = f (maxit huge, tolerance 0: every launch does full work)
    TOG_CUDA(cudaMemcpyAsync(h->d_r64, h->d_f, h->ndofs * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    if (precision == TOG_FP64) {
        launch_pcg_init<double>(h, h->stream, 1, 0.0, 0.0, h->fnorm2, 1 << 30);
        launch_matvec<double, MV_PCG>(h, h->stream, nullptr, nullptr, nullptr);
        for (int i = 0; i < nlaunch; ++i) {
            if (kernel == 0)
                launch_matvec<double, MV_PCG>(h, h->stream, nullptr, nullptr, nullptr);
            else
                launch_pcg_update<double>(h, h->stream);
        }
    } else {
        TOG_CUDA(cudaMemcpyAsync(&h->d_st64->rr, &h->fnorm2, sizeof(double), cudaMemcpyHostToDevice, h->stream));
        TOG_CUDA(cudaStreamSynchronize(h->stream));
        const int nb = h->ew_blocks(h->ndofs);
        if (h->dim == 3)
            k_ir_scale<3><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, h->ndofs, h->d_st64);
        else
            k_ir_scale<2><<<nb, kEwThreads, 0, h->stream>>>(h->d_r64, h->d_r32, h->ndofs, h->d_st64);
        TOG_LAUNCHED(1);
        launch_pcg_init<float>(h, h->stream, 1, 0.0, 0.0, -1.0, 1 << 30);
        launch_matvec<float, MV_PCG>(h, h->stream, nullptr, nullptr, nullptr);
        for (int i = 0; i < nlaunch; ++i) {
            if (kernel == 0)
                launch_matvec<float, MV_PCG>(h, h->stream, nullptr, nullptr, nullptr);
            else
                launch_pcg_update<float>(h, h->stream);
        }
    }
    TOG_CUDA(cudaGetLastError());
    return TOG_OK;
}

int tog_kernel_bytes(tog_handle* h, int32_t kernel, int32_t precision, double* bytes) {
    TOG_TRY(check_handle(h));
    if (!bytes || kernel < 0 || kernel > 1) return fail(TOG_ERR_ARG, "bad kernel id or null output");
    const double s = precision == TOG_FP64 ? 8.0 : 4.0;
    const double N = (double)h->ndofs, Nn = (double)h->nnodes, E = (double)h->ncells;
    const bool march = h->dim == 3 && precision != TOG_FP64;
    if (kernel == 0)   // reads r, p_old, D^-1, E_e (and the fixed mask, except the 3D march); writes p, q
        *bytes = 4.0 * s * N + s * Nn + s * E + (march ? 0.0 : Nn);
    else               // reads q, p, x, r, D^-1, mask; writes x, r
        *bytes = 6.0 * s * N + s * Nn + Nn;
    return TOG_OK;
}

}  // extern "C"
