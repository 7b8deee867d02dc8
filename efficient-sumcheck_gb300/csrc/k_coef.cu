// k_coef.cu -- round kernels of the CoefficientProver (product evaluator of
// degree 1..3, MSB and LSB).
#include "round_common.cuh"

namespace effsc {

#define EVAL(POL, SEM, M) \
    case ((POL) * 64 + (SEM) * 16 + (M)): return launch_chain(k_eval<POL, SEM, M>, grid, TPB, 0, s, a);

bool launch_eval_coef(int pol, int sem, u32 mask, const RoundArgs& a, int grid, cudaStream_t s) {
    switch (pol * 64 + sem * 16 + (int)mask) {
        EVAL(POL_C1, SEM_MSB_FLOOR, 0) EVAL(POL_C1, SEM_MSB_FLOOR, 1)
        EVAL(POL_C1, SEM_LSB, 0) EVAL(POL_C1, SEM_LSB, 1)
        EVAL(POL_C2, SEM_MSB_FLOOR, 0) EVAL(POL_C2, SEM_MSB_FLOOR, 3)
        EVAL(POL_C2, SEM_LSB, 0) EVAL(POL_C2, SEM_LSB, 3)
        EVAL(POL_C3, SEM_MSB_FLOOR, 0) EVAL(POL_C3, SEM_MSB_FLOOR, 1) EVAL(POL_C3, SEM_MSB_FLOOR, 7)
        EVAL(POL_C3, SEM_LSB, 0) EVAL(POL_C3, SEM_LSB, 1) EVAL(POL_C3, SEM_LSB, 7)
        EVAL(POL_C3W, SEM_MSB_FLOOR, 0) EVAL(POL_C3W, SEM_MSB_FLOOR, 1) EVAL(POL_C3W, SEM_MSB_FLOOR, 7)
        EVAL(POL_C3W, SEM_LSB, 0) EVAL(POL_C3W, SEM_LSB, 1) EVAL(POL_C3W, SEM_LSB, 7)
        default: return false;
    }
}

#define FUSED(POL, SEM, M, ECH) \
    case ((POL) * 128 + (SEM) * 32 + (M) * 2 + (ECH)): return launch_chain(k_fused<POL, SEM, M, ECH>, wave_grid<k_fused<POL, SEM, M, ECH>>(grid), TPB, 0, s, a);
#define FUSED_WIDE(POL, SEM, M, ECH) \
    case ((POL) * 128 + (SEM) * 32 + (M) * 2 + (ECH)): return launch_chain(k_fused_wide<POL, SEM, M, ECH>, wave_grid<k_fused_wide<POL, SEM, M, ECH>>(grid), TPB, 0, s, a);

bool launch_fused_coef(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    switch (pol * 128 + sem * 32 + (int)mask * 2 + (ech ? 1 : 0)) {
        FUSED(POL_C1, SEM_MSB_FLOOR, 0, false) FUSED(POL_C1, SEM_MSB_FLOOR, 0, true) FUSED(POL_C1, SEM_MSB_FLOOR, 1, true)
        FUSED(POL_C1, SEM_LSB, 0, false) FUSED(POL_C1, SEM_LSB, 0, true) FUSED(POL_C1, SEM_LSB, 1, true)
        FUSED(POL_C2, SEM_MSB_FLOOR, 0, false) FUSED(POL_C2, SEM_MSB_FLOOR, 0, true) FUSED(POL_C2, SEM_MSB_FLOOR, 3, true)
        FUSED(POL_C2, SEM_LSB, 0, false) FUSED(POL_C2, SEM_LSB, 0, true) FUSED(POL_C2, SEM_LSB, 3, true)
        FUSED_WIDE(POL_C3, SEM_MSB_FLOOR, 0, false) FUSED_WIDE(POL_C3, SEM_MSB_FLOOR, 0, true)
        FUSED_WIDE(POL_C3, SEM_MSB_FLOOR, 1, true) FUSED_WIDE(POL_C3, SEM_MSB_FLOOR, 7, true)
        FUSED_WIDE(POL_C3, SEM_LSB, 0, false) FUSED_WIDE(POL_C3, SEM_LSB, 0, true)
        FUSED_WIDE(POL_C3, SEM_LSB, 1, true) FUSED_WIDE(POL_C3, SEM_LSB, 7, true)
        FUSED_WIDE(POL_C3W, SEM_MSB_FLOOR, 0, false) FUSED_WIDE(POL_C3W, SEM_MSB_FLOOR, 0, true)
        FUSED_WIDE(POL_C3W, SEM_MSB_FLOOR, 1, true) FUSED_WIDE(POL_C3W, SEM_MSB_FLOOR, 7, true)
        FUSED_WIDE(POL_C3W, SEM_LSB, 0, false) FUSED_WIDE(POL_C3W, SEM_LSB, 0, true)
        FUSED_WIDE(POL_C3W, SEM_LSB, 1, true) FUSED_WIDE(POL_C3W, SEM_LSB, 7, true)
        default: return false;
    }
}

}  // namespace effsc
