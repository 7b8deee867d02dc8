// k_coef_expr.cu -- round polynomial of a CoefficientProver whose evaluator
// is given declaratively (ExprProgram, kernels.h): for every pair, each term
// multiplies its factors (even or odd elements of the columns) and adds the
// product into its term sum; the last block of the grid turns the term sums
// into the coefficients (times each term's constant) and the wire.  The
// columns are folded beforehand by the ordinary fold kernel, so this covers
// any evaluator of degree <= 3 whose accumulate_pair is a sum of constant
// multiples of products of pair elements (src/coefficient_sumcheck.rs:50-76;
// e.g. the reference's Degree1/Degree2/Mixed/InnerProduct test evaluators).
// Values are computed in Fp3 (base values embedded); a term sum is kept
// reduced (this path serves generality, the product evaluators have their
// own lazily accumulated kernels).
#include "round_common.cuh"

namespace effsc {

template <int SEM>
__global__ void __launch_bounds__(TPB) k_expr_eval(RoundArgs a, ExprProgram prog) {
    chain_enter();
    const u64 L = a.L, half = L / 2;
    F3 sums[EXPR_MAX_TERMS];
    for (u32 t = 0; t < prog.nterms; t++) sums[t] = f3_zero();
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    for (u64 j = tid; j < half; j += stride) {
        const u64 ilo = SEM == SEM_LSB ? 2 * j : j, ihi = SEM == SEM_LSB ? 2 * j + 1 : j + half;
        F3 v[8];
        for (u32 c = 0; c < prog.ncols; c++) {
            const bool e = a.t[c].in[1] != nullptr;
            v[2 * c] = e ? ld<true>(a.t[c].in, ilo) : ld<false>(a.t[c].in, ilo);
            v[2 * c + 1] = e ? ld<true>(a.t[c].in, ihi) : ld<false>(a.t[c].in, ihi);
        }
        for (u32 t = 0; t < prog.nterms; t++) {
            const ExprTerm& T = prog.t[t];
            F3 p = f3_make(1, 0, 0);
            for (u32 f = 0; f < T.nf; f++) p = f3_mul<true, true>(p, v[T.f[f]]);
            sums[t] = f3_add<true>(sums[t], p);
        }
    }
    // coefficient c = sum over its terms of k * (term sum)
    F3 raw[4];
    for (int c = 0; c < 4; c++) raw[c] = f3_zero();
    for (u32 t = 0; t < prog.nterms; t++) {
        const ExprTerm& T = prog.t[t];
        const F3 kt = f3_make(T.k[0], T.k[1], T.k[2]);
        const F3 x = f3_mul<true, true>(sums[t], kt);
        for (int c = 0; c < 4; c++)
            if (T.coeff == c) raw[c] = f3_add<true>(raw[c], x);
    }
    const int pol = prog.degree <= 1 ? POL_X1 : prog.degree == 2 ? POL_X2 : POL_X3;
    reduce_and_finalize<4>(raw, a, pol);
}

bool launch_expr_eval(int sem, const RoundArgs& a, const ExprProgram& prog, int grid, cudaStream_t s) {
    if (sem == SEM_LSB) return launch_chain(k_expr_eval<SEM_LSB>, grid, TPB, 0, s, a, prog);
    if (sem == SEM_MSB_FLOOR) return launch_chain(k_expr_eval<SEM_MSB_FLOOR>, grid, TPB, 0, s, a, prog);
    return false;
}

}  // namespace effsc
