// k_mlip.cu -- round kernels of the Multilinear, InnerProduct and EqFactored
// provers (template instantiations and their launch dispatch).
#include "round_common.cuh"

#include <atomic>

namespace effsc {

#define EVAL(POL, SEM, M) \
    case ((POL) * 64 + (SEM) * 16 + (M)): return launch_chain(k_eval<POL, SEM, M>, grid, TPB, 0, s, a);

bool launch_eval_mlip(int pol, int sem, u32 mask, const RoundArgs& a, int grid, cudaStream_t s) {
    switch (pol * 64 + sem * 16 + (int)mask) {
        EVAL(POL_ML, SEM_MSB_PAD, 0) EVAL(POL_ML, SEM_MSB_PAD, 1)
        EVAL(POL_ML, SEM_LSB, 0) EVAL(POL_ML, SEM_LSB, 1)
        EVAL(POL_IP, SEM_MSB_PAD, 0) EVAL(POL_IP, SEM_MSB_PAD, 3)
        EVAL(POL_IP, SEM_LSB, 0) EVAL(POL_IP, SEM_LSB, 3)
        EVAL(POL_EQFR, SEM_MSB_PAD, 0) EVAL(POL_EQFR, SEM_MSB_PAD, 1) EVAL(POL_EQFR, SEM_MSB_PAD, 3)
        default: return false;
    }
}

#define FUSED(POL, SEM, M, ECH) \
    case ((POL) * 128 + (SEM) * 32 + (M) * 2 + (ECH)): return launch_chain(k_fused<POL, SEM, M, ECH>, wave_grid<k_fused<POL, SEM, M, ECH>>(grid), TPB, 0, s, a);

bool launch_fused_mlip(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    switch (pol * 128 + sem * 32 + (int)mask * 2 + (ech ? 1 : 0)) {
        FUSED(POL_ML, SEM_MSB_PAD, 0, false) FUSED(POL_ML, SEM_MSB_PAD, 0, true) FUSED(POL_ML, SEM_MSB_PAD, 1, true)
        FUSED(POL_ML, SEM_LSB, 0, false) FUSED(POL_ML, SEM_LSB, 0, true) FUSED(POL_ML, SEM_LSB, 1, true)
        FUSED(POL_IP, SEM_MSB_PAD, 0, false) FUSED(POL_IP, SEM_MSB_PAD, 0, true) FUSED(POL_IP, SEM_MSB_PAD, 3, true)
        FUSED(POL_IP, SEM_LSB, 0, false) FUSED(POL_IP, SEM_LSB, 0, true) FUSED(POL_IP, SEM_LSB, 3, true)
        FUSED(POL_EQFR, SEM_MSB_PAD, 0, false) FUSED(POL_EQFR, SEM_MSB_PAD, 0, true)
        FUSED(POL_EQFR, SEM_MSB_PAD, 1, true) FUSED(POL_EQFR, SEM_MSB_PAD, 3, true)
        default: return false;
    }
}

template <int POL, int SEM, u32 M, bool ECH>
static bool launch_tma_inst(const RoundArgs& a, u32 ntiles, int grid, cudaStream_t s) {
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr int SM_BYTES = TmaLayout<M, NT>::smem_bytes();
    // the shared-memory limit is a per-device function attribute: set once
    // per device (one bit each), safe when threads race to set it
    static std::atomic<uint64_t> configured{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    const uint64_t bit = 1ull << (dev & 63);
    if (!(configured.load() & bit)) {
        if (cudaFuncSetAttribute(k_fused_tma<POL, SEM, M, ECH>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_BYTES) != cudaSuccess)
            return false;
        configured.fetch_or(bit);
    }
    return launch_chain(k_fused_tma<POL, SEM, M, ECH>, grid, TPB, SM_BYTES, s, a, ntiles);
}

bool launch_fused_tma(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, u32 ntiles, int grid, cudaStream_t s) {
    int key = pol * 64 + (sem == SEM_LSB ? 32 : 0) + (int)mask * 2 + (ech ? 1 : 0);
    switch (key) {
        case POL_IP * 64 + 0 * 2 + 0: return launch_tma_inst<POL_IP, SEM_MSB_PAD, 0, false>(a, ntiles, grid, s);
        case POL_IP * 64 + 0 * 2 + 1: return launch_tma_inst<POL_IP, SEM_MSB_PAD, 0, true>(a, ntiles, grid, s);
        case POL_IP * 64 + 3 * 2 + 1: return launch_tma_inst<POL_IP, SEM_MSB_PAD, 3, true>(a, ntiles, grid, s);
        case POL_IP * 64 + 32 + 0 * 2 + 0: return launch_tma_inst<POL_IP, SEM_LSB, 0, false>(a, ntiles, grid, s);
        case POL_IP * 64 + 32 + 0 * 2 + 1: return launch_tma_inst<POL_IP, SEM_LSB, 0, true>(a, ntiles, grid, s);
        case POL_IP * 64 + 32 + 3 * 2 + 1: return launch_tma_inst<POL_IP, SEM_LSB, 3, true>(a, ntiles, grid, s);
        default: return false;
    }
}
int fused_tma_blocks_per_sm(void) { return 2; }

bool launch_eqf_left(bool fused, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    int key = (fused ? 16 : 0) + (int)mask * 2 + (ech ? 1 : 0);
    switch (key) {
        case 0 + 0 * 2 + 0: k_eqf_left<false, 0, false><<<grid, TPB, 0, s>>>(a); return true;
        case 0 + 2 * 2 + 0: k_eqf_left<false, 2, false><<<grid, TPB, 0, s>>>(a); return true;
        case 0 + 3 * 2 + 0: k_eqf_left<false, 3, false><<<grid, TPB, 0, s>>>(a); return true;
        case 16 + 0 * 2 + 0: k_eqf_left<true, 0, false><<<grid, TPB, 0, s>>>(a); return true;
        case 16 + 0 * 2 + 1: k_eqf_left<true, 0, true><<<grid, TPB, 0, s>>>(a); return true;
        case 16 + 2 * 2 + 1: k_eqf_left<true, 2, true><<<grid, TPB, 0, s>>>(a); return true;
        case 16 + 3 * 2 + 1: k_eqf_left<true, 3, true><<<grid, TPB, 0, s>>>(a); return true;
        default: return false;
    }
}

}  // namespace effsc
