// ml01.cuh -- two-pass start of an MSB Multilinear proof (rounds 0-1 from
// one pass, round 2 with a double fold from a second), the Multilinear
// counterpart of ip01.cuh.
//
// With quarters S_j = sum_k v[k + jQ] (Q = L/4) of the table, round 0's wire
// is s0 = S_0 + S_1 and, since every entry of the table folded with r0 is
// linear in r0, round 1's is s0' = S_0 + r0 (S_2 - S_0)
// (src/multilinear_sumcheck.rs:86-124 on the folded table).  The first pass
// reads three quarters of the table once and its last block runs both
// transcript steps; the second folds with r0 and r1 at once,
//   v''[k] = x0 + r0 (x2 - x0) + r1 (x1 - x0) + r0 r1 (x3 - x2 - x1 + x0),
// x_j = v[k + jQ], writes the length-L/4 table and evaluates round 2 on it.
#pragma once
#include "ip01.cuh"

namespace effsc {

__device__ __forceinline__ void ml01_body(const RoundArgs& a, u32 bid, u32 nb) {
    Acc s0 = acc_zero(), s1 = acc_zero(), s2 = acc_zero();
    const u64 Q = a.L >> 2;
    const u64* X = a.t[0].in[0];
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    for (u64 k = tid; k < Q; k += stride) {
        acc_add64(s0, __ldcs(X + k));
        acc_add64(s1, __ldcs(X + k + Q));
        acc_add64(s2, __ldcs(X + k + 2 * Q));
    }
    F3 raw[1] = {f3_make(acc_reduce(s0), acc_reduce(s1), acc_reduce(s2))};
    reduce_and_finalize_seg<1>(raw, a, POL_ML01, nb, bid);
}

// v''[k] with base challenges (one reduction) or Fp3 ones (fold2).
template <bool ECH>
__device__ __forceinline__ F3 ml_fold2(u64 x0, u64 x1, u64 x2, u64 x3, const F3& r0, const F3& r1, const F3& r01) {
    if (ECH) return fold2(x0, x1, x2, x3, r0, r1, r01);
    const u64 d1 = gl_sub(x2, x0), d2 = gl_sub(x1, x0), d3 = gl_sub(gl_sub(x3, x2), d2);
    Acc c = acc_from(x0);
    acc_mac(c, d1, r0.c0);
    acc_mac(c, d2, r1.c0);
    acc_mac(c, d3, r01.c0);
    return f3_make(acc_reduce(c), 0, 0);
}

template <bool ECH>
__device__ __forceinline__ void ml2x_body(const RoundArgs& a, u32 bid, u32 nb) {
    using P = Policy<POL_ML, ECH ? 1u : 0u>;
    P acc;
    acc.init();
    const F3 r0 = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    const F3 r1 = f3_make(a.chal2_ptr[0], a.chal2_ptr[1], a.chal2_ptr[2]);
    const F3 r01 = f3_mul<ECH, ECH>(r0, r1);
    const u64 Q = a.L >> 2, H = Q >> 1;   // v'' has Q entries; round 2 pairs (m, m + H)
    const u64* X = a.t[0].in[0];
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    F3 lo[1], hi[1];
    for (u64 m = tid; m < H; m += stride) {
        lo[0] = ml_fold2<ECH>(__ldcs(X + m), __ldcs(X + m + Q), __ldcs(X + m + 2 * Q), __ldcs(X + m + 3 * Q), r0, r1, r01);
        hi[0] = ml_fold2<ECH>(__ldcs(X + m + H), __ldcs(X + m + H + Q), __ldcs(X + m + H + 2 * Q), __ldcs(X + m + H + 3 * Q),
                              r0, r1, r01);
        st<ECH>(a.t[0].out, m, lo[0]);
        st<ECH>(a.t[0].out, m + H, hi[0]);
        acc.pair(lo, hi);
    }
    F3 raw[2];
    acc.result(raw);
    reduce_and_finalize_seg<2>(raw, a, POL_ML, nb, bid);
}

}  // namespace effsc
