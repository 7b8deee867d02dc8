// k_ip01.cu -- single-instance kernels of the two-pass starts: MSB / LSB
// InnerProduct over Fp3 challenges (bodies in ip01.cuh) and MSB Multilinear
// (ml01.cuh).
#include "ml01.cuh"

namespace effsc {

template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r01(RoundArgs a) { ip01_body<LSB>(a, blockIdx.x, gridDim.x); }
template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r2x(RoundArgs a) { ip2x_body<LSB>(a, blockIdx.x, gridDim.x); }

bool launch_ip01(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    if (lsb) k_ip_r01<true><<<grid, TPB, 0, s>>>(a);
    else k_ip_r01<false><<<grid, TPB, 0, s>>>(a);
    return true;
}
bool launch_ip2x(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    if (lsb) k_ip_r2x<true><<<grid, TPB, 0, s>>>(a);
    else k_ip_r2x<false><<<grid, TPB, 0, s>>>(a);
    return true;
}

__global__ void __launch_bounds__(TPB, 2) k_ml_r01(RoundArgs a) { ml01_body(a, blockIdx.x, gridDim.x); }
template <bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_ml_r2x(RoundArgs a) { ml2x_body<ECH>(a, blockIdx.x, gridDim.x); }

bool launch_ml01(const RoundArgs& a, int grid, cudaStream_t s) {
    k_ml_r01<<<grid, TPB, 0, s>>>(a);
    return true;
}
bool launch_ml2x(bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    if (ech) k_ml_r2x<true><<<grid, TPB, 0, s>>>(a);
    else k_ml_r2x<false><<<grid, TPB, 0, s>>>(a);
    return true;
}

}  // namespace effsc
