// k_coef01.cu -- single-instance kernels of the Coefficient (degree-3 product
// evaluator) start that runs rounds 0-2 in two passes (bodies in coef01.cuh).
#include "coef01.cuh"

namespace effsc {

template <bool LSB, bool E0>
__global__ void __launch_bounds__(TPB, 2) k_c3_r01(RoundArgs a) {
    chain_enter();
    c301_body<LSB, E0>(a, blockIdx.x, gridDim.x);
}
template <bool LSB, bool E0>
__global__ void __launch_bounds__(TPB, 2) k_c3_r2x(RoundArgs a) {   // spills a little; measured faster than one block per SM
    chain_enter();
    c32x_body<LSB, E0>(a, blockIdx.x, gridDim.x);
}

bool launch_c3_r01(bool lsb, bool e0, const RoundArgs& a, int grid, cudaStream_t s) {
    if (lsb) return e0 ? launch_chain(k_c3_r01<true, true>, grid, TPB, 0, s, a) : launch_chain(k_c3_r01<true, false>, grid, TPB, 0, s, a);
    return e0 ? launch_chain(k_c3_r01<false, true>, grid, TPB, 0, s, a) : launch_chain(k_c3_r01<false, false>, grid, TPB, 0, s, a);
}
#define C3X(LSB, E0) launch_chain(k_c3_r2x<LSB, E0>, wave_grid<k_c3_r2x<LSB, E0>>(grid), TPB, 0, s, a)
bool launch_c3_r2x(bool lsb, bool e0, const RoundArgs& a, int grid, cudaStream_t s) {
    if (lsb) return e0 ? C3X(true, true) : C3X(true, false);
    return e0 ? C3X(false, true) : C3X(false, false);
}
#undef C3X

}  // namespace effsc
