// k_ip012.cu -- single-instance kernels of the InnerProduct start that runs
// rounds 0-3 in two passes (bodies in ip012.cuh).
#include "ip012.cuh"

#include <atomic>

namespace effsc {

template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r012(RoundArgs a) {
    chain_enter();
    ip012_body<LSB>(a, blockIdx.x, gridDim.x);
}
template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r012m(RoundArgs a) {
    chain_enter();
    ip012_body<LSB, true>(a, blockIdx.x, gridDim.x);
}
template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r3x(RoundArgs a) {
    chain_enter();
    ip3x_body<LSB>(a, blockIdx.x, gridDim.x);
}

template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r012s(RoundArgs a, u32 ntiles) {
    chain_enter();
    ip012_staged_body<LSB>(a, ntiles);
}

// The dynamic shared-memory limit is a per-device function attribute: set
// once per device (one bit each), safe when threads race to set it.
template <class K>
static bool allow_smem(K kernel, int bytes, std::atomic<uint64_t>& configured) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    const uint64_t bit = 1ull << (dev & 63);
    if (!(configured.load() & bit)) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return false;
        configured.fetch_or(bit);
    }
    return true;
}

bool launch_ip012_staged(bool lsb, const RoundArgs& a, u32 ntiles, int grid, cudaStream_t s) {
    static std::atomic<uint64_t> cfg[2];
    if (lsb) {
        if (!allow_smem(k_ip_r012s<true>, IP012_SMEM, cfg[1])) return false;
        return launch_chain(k_ip_r012s<true>, grid, TPB, IP012_SMEM, s, a, ntiles);
    }
    if (!allow_smem(k_ip_r012s<false>, IP012_SMEM, cfg[0])) return false;
    return launch_chain(k_ip_r012s<false>, grid, TPB, IP012_SMEM, s, a, ntiles);
}
u32 ip012_tile_octets(void) { return IP012_TQ; }

bool launch_ip012_mirror(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    return lsb ? launch_chain(k_ip_r012m<true>, grid, TPB, 0, s, a) : launch_chain(k_ip_r012m<false>, grid, TPB, 0, s, a);
}
bool launch_ip012(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    return lsb ? launch_chain(k_ip_r012<true>, grid, TPB, 0, s, a) : launch_chain(k_ip_r012<false>, grid, TPB, 0, s, a);
}
bool launch_ip3x(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    return lsb ? launch_chain(k_ip_r3x<true>, grid, TPB, 0, s, a) : launch_chain(k_ip_r3x<false>, grid, TPB, 0, s, a);
}

}  // namespace effsc
