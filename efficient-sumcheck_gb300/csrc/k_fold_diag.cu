// k_fold_diag.cu -- diagnostics.  The transcript latency probe times the
// warp-wide permutation and one transcript round step.  The self-test of the
// bounded wait used by the TMA-staged round kernel: one thread waits on a shared-memory mbarrier that nothing
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

// Latency of the transcript on one warp: `iters` permutations back to back,
// then `iters` round steps (send one Fp3 element, squeeze one challenge), each
// timed with the global timer; out = {ns per permutation, ns per step}.
__global__ void k_diag_transcript(u32 iters, u64* out) {
    __shared__ u64 s_v[3], s_chal[3];
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x;
    WarpTx w;
    w.a = lane < 25 ? (u64)lane * 0x9E3779B97F4A7C15ULL : 0;
    w.pos = 0;
    w.squeezing = 0;
    w.deg = 3;
    if (lane < 3) s_v[lane] = 1 + lane;
    __syncwarp();
    const u64 t0 = global_ns();
    for (u32 k = 0; k < iters; k++) keccak_f_warp(w.a, lane);
    const u64 t1 = global_ns();
    for (u32 k = 0; k < iters; k++) {
        tx_send_elems(w, lane, s_v, 1);
        tx_challenge(w, lane, s_chal, s_scr);
        if (lane < 3) s_v[lane] = s_chal[lane];
        __syncwarp();
    }
    const u64 t2 = global_ns();
    if (lane == 0) {
        out[0] = (t1 - t0) / iters;
        out[1] = (t2 - t1) / iters;
        out[2] = w.a;   // keeps the work observable
    }
}

void launch_diag_transcript(u32 iters, u64* out, cudaStream_t s) { k_diag_transcript<<<1, 32, 0, s>>>(iters, out); }

}  // namespace effsc
