// k_ip01.cu -- single-instance kernels of the two-pass starts: MSB / LSB
// InnerProduct over Fp3 challenges (bodies in ip01.cuh) and MSB Multilinear
// (ml01.cuh).
#include "ml01.cuh"

namespace effsc {

template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r01(RoundArgs a) {
    chain_enter();
    ip01_body<LSB>(a, blockIdx.x, gridDim.x);
}
template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r2x(RoundArgs a) {
    chain_enter();
    ip2x_body<LSB>(a, blockIdx.x, gridDim.x);
}

bool launch_ip01(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    return lsb ? launch_chain(k_ip_r01<true>, grid, TPB, 0, s, a) : launch_chain(k_ip_r01<false>, grid, TPB, 0, s, a);
}
bool launch_ip2x(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    return lsb ? launch_chain(k_ip_r2x<true>, grid, TPB, 0, s, a) : launch_chain(k_ip_r2x<false>, grid, TPB, 0, s, a);
}

__global__ void __launch_bounds__(TPB, 2) k_ml_r01(RoundArgs a) {
    chain_enter();
    ml01_body(a, blockIdx.x, gridDim.x);
}
template <bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_ml_r2x(RoundArgs a) {
    chain_enter();
    ml2x_body<ECH>(a, blockIdx.x, gridDim.x);
}

bool launch_ml01(const RoundArgs& a, int grid, cudaStream_t s) {
    return launch_chain(k_ml_r01, grid, TPB, 0, s, a);
}
bool launch_ml2x(bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    return ech ? launch_chain(k_ml_r2x<true>, grid, TPB, 0, s, a) : launch_chain(k_ml_r2x<false>, grid, TPB, 0, s, a);
}

}  // namespace effsc
