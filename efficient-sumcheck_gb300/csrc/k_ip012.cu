// k_ip012.cu -- single-instance kernels of the InnerProduct start that runs
// rounds 0-3 in two passes (bodies in ip012.cuh).
#include "ip012.cuh"

namespace effsc {

template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r012(RoundArgs a) { ip012_body<LSB>(a, blockIdx.x, gridDim.x); }
template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_r3x(RoundArgs a) { ip3x_body<LSB>(a, blockIdx.x, gridDim.x); }

bool launch_ip012(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    if (lsb) k_ip_r012<true><<<grid, TPB, 0, s>>>(a);
    else k_ip_r012<false><<<grid, TPB, 0, s>>>(a);
    return true;
}
bool launch_ip3x(bool lsb, const RoundArgs& a, int grid, cudaStream_t s) {
    if (lsb) k_ip_r3x<true><<<grid, TPB, 0, s>>>(a);
    else k_ip_r3x<false><<<grid, TPB, 0, s>>>(a);
    return true;
}

}  // namespace effsc
