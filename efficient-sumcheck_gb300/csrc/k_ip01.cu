// k_ip01.cu -- single-instance kernels of the two-pass start of an MSB
// InnerProduct proof over Fp3 challenges (bodies in ip01.cuh).
#include "ip01.cuh"

namespace effsc {

__global__ void __launch_bounds__(TPB, 2) k_ip_r01(RoundArgs a) { ip01_body(a, blockIdx.x, gridDim.x); }
__global__ void __launch_bounds__(TPB, 2) k_ip_r2x(RoundArgs a) { ip2x_body(a, blockIdx.x, gridDim.x); }

bool launch_ip01(const RoundArgs& a, int grid, cudaStream_t s) {
    k_ip_r01<<<grid, TPB, 0, s>>>(a);
    return true;
}
bool launch_ip2x(const RoundArgs& a, int grid, cudaStream_t s) {
    k_ip_r2x<<<grid, TPB, 0, s>>>(a);
    return true;
}

}  // namespace effsc
