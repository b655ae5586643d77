// Checks the bounded mbarrier wait of the tcgen05 kernels (topopt.jl_gb300/csrc/tog_tc.cuh)
// without a GPU fault: one block allocates TMEM, waits with a small poll limit on an
// mbarrier that nothing arrives on, must see the wait give up, frees its TMEM and reports;
// a second block waits on an mbarrier that one of its threads arrives on and must see it
// complete.  The context stays usable: a third launch runs after both.  Prints
// "timeout=<0|1> completed=<0|1> after=<0|1>" and exits 0 when they are 1 1 1.
#include <cstdio>
#include "../topopt.jl_gb300/csrc/tog_tc.cuh"

using namespace tog;

__global__ void k_wait(int arrive, int limit, int* out) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(&slot, 32);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (arrive && tid == 0) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(&bar)) : "memory");
    }
    const bool done = tc::mbar_wait(&bar, 0, limit);
    const bool all = __syncthreads_and(done);
    const bool none = !__syncthreads_or(done);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(slot, 32);
    }
    if (tid == 0) *out = arrive ? (all ? 1 : 0) : (none ? 1 : 0);
}

__global__ void k_after(int* out) { *out = 1; }

int main() {
    int* d;
    if (cudaMalloc(&d, 3 * sizeof(int)) != cudaSuccess) return 2;
    cudaMemset(d, 0, 3 * sizeof(int));
    k_wait<<<1, 128>>>(0, 2000, d);        // nothing arrives: the wait must give up
    k_wait<<<1, 128>>>(1, 1 << 20, d + 1);   // thread 0 arrives: the wait must complete
    k_after<<<1, 1>>>(d + 2);
    const cudaError_t e = cudaDeviceSynchronize();
    int h[3] = {0, 0, 0};
    cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    printf("timeout=%d completed=%d after=%d cuda=%s\n", h[0], h[1], h[2], cudaGetErrorString(e));
    return (e == cudaSuccess && h[0] == 1 && h[1] == 1 && h[2] == 1) ? 0 : 1;
}
