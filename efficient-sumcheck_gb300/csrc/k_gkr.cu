// k_gkr.cu -- GkrProver rounds (src/provers/gkr.rs:105-190).
//
// The reference expands the witness into two broadcast tables of 2^(2k)
// entries, w_b[b n + c] = W(b) and w_c[b n + c] = W(c), and folds all four
// tables every round.  Folding w_c over a b variable leaves it unchanged and
// folding w_b over a c variable likewise, so here the witness stays two
// compact tables: W_b (folded during the first k rounds) and W_c (folded
// during the last k); entry i of the current gate tables reads
//   W_b[i >> kc] and W_c[i & (2^kc - 1)],  kc = min(k, log2 |add|),
// the same values the broadcast tables hold.  Each round evaluates
// f(x) = add (W_b + W_c) + mult W_b W_c at x = 0, 1, 2 over the pairs
// (i, i + half) -- optionally right after folding add and mult with the
// previous challenge in the same pass -- and the last block turns the three
// sums into the wire [q(0), (q(0) + q(2) - 2 q(1)) / 2].
#include "round_common.cuh"

namespace effsc {

// W_b and W_c keep their own representation: W_c stays in the base field
// through the first k rounds (it is folded only in the last k) and W_b is
// base in round 0, so the W sum and product are mixed or base there.
template <bool EA, bool EWB, bool EWC>
__device__ __forceinline__ void gkr_point(ProdAcc<EA, EWB || EWC>& acc, const F3& a, const F3& m, const F3& wb,
                                          const F3& wc) {
    acc.mac(a, f3_add_mixed<EWB || EWC, EWB && EWC>(EWB || !EWC ? wb : wc, EWB || !EWC ? wc : wb));
    acc.mac(m, f3_mul<EWB, EWC>(wb, wc));
}

template <bool E>
__device__ __forceinline__ F3 twice_minus(const F3& hi, const F3& lo) {
    return f3_sub<E>(f3_add<E>(hi, hi), lo);
}

// Blocks per SM the register budget is sized for: Fp3 gate tables with an
// Fp3 witness keep three Fp3 x Fp3 accumulators (75 registers) live, which
// fit without spills only at one block per SM.
template <bool FUSED, bool EAI, bool EWB, bool EWC, bool ECH>
constexpr int gkr_min_blocks() { return ((FUSED ? (EAI || ECH) : EAI) && (EWB || EWC)) ? 1 : 2; }

template <bool FUSED, bool EAI, bool EWB, bool EWC, bool ECH>
__global__ void __launch_bounds__(TPB, (gkr_min_blocks<FUSED, EAI, EWB, EWC, ECH>())) k_gkr(RoundArgs a) {
    constexpr bool EA = FUSED ? (EAI || ECH) : EAI;   // add / mult after the fold
    constexpr bool EW = EWB || EWC;
    ProdAcc<EA, EW> q0, q1, q2;
    q0.init();
    q1.init();
    q2.init();
    const u64 L = a.L;
    const u64 Ln = FUSED ? L >> 1 : L;                 // length evaluated
    const u32 lg = 63 - __clzll(Ln > 0 ? Ln : 1);
    const u32 kc = a.m_shift < lg ? a.m_shift : lg;
    const u64 cm = (1ULL << kc) - 1;
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    if (Ln == 1) {
        if (tid == 0) {
            const F3 al = ld<EA>(FUSED ? (const u64* const*)a.t[0].out : a.t[0].in, 0);
            const F3 ml = ld<EA>(FUSED ? (const u64* const*)a.t[1].out : a.t[1].in, 0);
            const F3 wb = ld<EWB>(a.t[2].in, 0), wc = ld<EWC>(a.t[3].in, 0);
            gkr_point<EA, EWB, EWC>(q0, al, ml, wb, wc);
            // q(2) = -q(0) so that the wire's q(inf) is 0 (src/provers/gkr.rs:119-127)
            gkr_point<EA, EWB, EWC>(q2, f3_sub<EA>(f3_zero(), al), f3_sub<EA>(f3_zero(), ml), wb, wc);
        }
    } else {
        F3 rr;
        Mul3 r = load_challenge_mul(a, rr);
        if (!ECH) r = mul3_prepare<false>(rr);
        const u64 H = Ln >> 1;
        for (u64 i = tid; i < H; i += stride) {
            F3 al, ah, ml, mh;
            if (FUSED) {
                F3 x[2][4];
#pragma unroll
                for (int t = 0; t < 2; t++)
#pragma unroll
                    for (int j = 0; j < 4; j++) x[t][j] = ld<EAI>(a.t[t].in, i + j * H);
                F3 lo[2], hi[2];
#pragma unroll
                for (int t = 0; t < 2; t++) {
                    if (EAI) { lo[t] = f3_fold<true, true>(x[t][0], x[t][2], r); hi[t] = f3_fold<true, true>(x[t][1], x[t][3], r); }
                    else if (ECH) { lo[t] = f3_fold<false, true>(x[t][0], x[t][2], r); hi[t] = f3_fold<false, true>(x[t][1], x[t][3], r); }
                    else { lo[t] = f3_fold<false, false>(x[t][0], x[t][2], r); hi[t] = f3_fold<false, false>(x[t][1], x[t][3], r); }
                    st<EA>(a.t[t].out, i, lo[t]);
                    st<EA>(a.t[t].out, i + H, hi[t]);
                }
                al = lo[0]; ah = hi[0]; ml = lo[1]; mh = hi[1];
            } else {
                al = ld<EA>(a.t[0].in, i); ah = ld<EA>(a.t[0].in, i + H);
                ml = ld<EA>(a.t[1].in, i); mh = ld<EA>(a.t[1].in, i + H);
            }
            const F3 wbl = ld<EWB>(a.t[2].in, i >> kc), wbh = ld<EWB>(a.t[2].in, (i + H) >> kc);
            const F3 wcl = ld<EWC>(a.t[3].in, i & cm), wch = ld<EWC>(a.t[3].in, (i + H) & cm);
            gkr_point<EA, EWB, EWC>(q0, al, ml, wbl, wcl);
            gkr_point<EA, EWB, EWC>(q1, ah, mh, wbh, wch);
            gkr_point<EA, EWB, EWC>(q2, twice_minus<EA>(ah, al), twice_minus<EA>(mh, ml), twice_minus<EWB>(wbh, wbl),
                                    twice_minus<EWC>(wch, wcl));
        }
    }
    F3 raw[3] = {q0.result(), q1.result(), q2.result()};
    reduce_and_finalize<3>(raw, a, POL_GKR);
}

#define GKR(F, EA, EWB, EWC, ECH) \
    case ((F) * 16 + (EA) * 8 + (EWB) * 4 + (EWC) * 2 + (ECH)): k_gkr<F, EA, EWB, EWC, ECH><<<grid, TPB, 0, s>>>(a); return true;

bool launch_gkr(bool fused, bool ea, bool ewb, bool ewc, bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    switch ((fused ? 16 : 0) + (ea ? 8 : 0) + (ewb ? 4 : 0) + (ewc ? 2 : 0) + (ech ? 1 : 0)) {
        // evaluate only (round 0, tables of length <= 2)
        GKR(false, false, false, false, false) GKR(false, false, true, false, false)
        GKR(false, false, false, true, false) GKR(false, false, true, true, false)
        GKR(false, true, false, false, false) GKR(false, true, true, false, false)
        GKR(false, true, false, true, false) GKR(false, true, true, true, false)
        // fused fold + evaluate: base challenges, or Fp3 challenges
        GKR(true, false, false, false, false)
        GKR(true, false, false, false, true) GKR(true, false, true, false, true)
        GKR(true, false, false, true, true) GKR(true, false, true, true, true)
        GKR(true, true, false, false, true) GKR(true, true, true, false, true)
        GKR(true, true, false, true, true) GKR(true, true, true, true, true)
        default: return false;
    }
}

}  // namespace effsc
