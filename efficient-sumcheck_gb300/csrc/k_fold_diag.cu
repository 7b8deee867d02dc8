// k_fold_diag.cu -- self-test of the bounded wait used by the TMA-staged
// round kernel: one thread waits on a shared-memory mbarrier that nothing
// completes (or that it completes itself first) with a short limit, and
// reports through a status word whether the wait gave up.  No other block,
// kernel or host action is involved, so the kernel always returns.
#include "round_common.cuh"

namespace effsc {

__global__ void k_diag_bounded_wait(u64 limit_ns, int arrive, u32* status) {
    __shared__ __align__(8) u64 bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
    const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
    *(volatile u32*)status = ok ? 0u : EFFSC_STATUS_TIMEOUT;
}

void launch_diag_bounded_wait(u64 limit_ns, int arrive, u32* status, cudaStream_t s) {
    k_diag_bounded_wait<<<1, 32, 0, s>>>(limit_ns, arrive, status);
}

}  // namespace effsc
