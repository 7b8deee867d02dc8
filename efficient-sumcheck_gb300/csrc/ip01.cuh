// ip01.cuh -- bodies of the two-pass start of an MSB InnerProduct proof over
// Fp3 challenges (rounds 0-1 from one pass, round 2 with a double fold from a
// second); used by the single-instance kernels (k_ip01.cu) and by the
// batched / serving step kernels.
//
// Round 1 evaluates the tables folded with r0, and each folded entry is
// linear in r0, so round 1's two sums are quadratics in r0 whose six
// base-field coefficients can be accumulated during round 0's pass
// (finalize_ip01 in round_common.cuh lists them).  The last block of that
// pass produces round 0's and round 1's wire values and both challenges.
// The second pass reads the base tables again, folds with r0 and then r1
// (new = lo + (hi - lo) r, src/inner_product_sumcheck.rs:143-176), writes the
// Fp3 tables of length L/4 and evaluates round 2 on them.  Compared with
// rounds 0, 1, 2 as separate passes this skips writing and re-reading the
// length-L/2 Fp3 tables (40 bytes per entry of L) and computes the same
// field values.
#pragma once
#include "round_common.cuh"

namespace effsc {

// Pass 1: quadruples (k, k+Q, k+2Q, k+3Q), Q = L/4, of both base tables;
// two quadruples per iteration so that sixteen loads are in flight.
__device__ __forceinline__ void ip01_quad(Acc (&s)[8], u64 a0, u64 a1, u64 a2, u64 a3, u64 b0, u64 b1, u64 b2, u64 b3) {
    const u64 da = gl_sub(a2, a0), db = gl_sub(b2, b0);
    const u64 da1 = gl_sub(a3, a1), db1 = gl_sub(b3, b1);
    const u64 ea = gl_sub(a1, a0), eb = gl_sub(b1, b0);
    const u64 fa = gl_sub(da1, da), fb = gl_sub(db1, db);
    acc_mac(s[0], a0, b0);
    acc_mac(s[1], a0, db);
    acc_mac(s[1], da, b0);
    acc_mac(s[2], da, db);
    acc_mac(s[3], ea, eb);
    acc_mac(s[4], ea, fb);
    acc_mac(s[4], fa, eb);
    acc_mac(s[5], fa, fb);
    acc_mac(s[6], a1, b1);
    acc_mac(s[7], da1, db1);
}

// LSB (pairs 2k, 2k+1, src/provers/inner_product_lsb.rs): quadruple k is
// entries 4k .. 4k+3; round 0 pairs (4k, 4k+1), (4k+2, 4k+3) and round 1
// pairs their folds, so it is the MSB quadruple with its middle two entries
// exchanged.
template <bool LSB>
__device__ __forceinline__ void ip01_body(const RoundArgs& a, u32 bid, u32 nb) {
    Acc s[8];
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = acc_zero();
    const u64 Q = a.L >> 2;
    const u64* A = a.t[0].in[0];
    const u64* B = a.t[1].in[0];
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    u64 k = tid;
    if (LSB) {
        const ulonglong2* A2 = (const ulonglong2*)A;
        const ulonglong2* B2 = (const ulonglong2*)B;
        for (; k < Q; k += stride) {
            const ulonglong2 xa = __ldcs(A2 + 2 * k), ya = __ldcs(A2 + 2 * k + 1);
            const ulonglong2 xb = __ldcs(B2 + 2 * k), yb = __ldcs(B2 + 2 * k + 1);
            ip01_quad(s, xa.x, ya.x, xa.y, ya.y, xb.x, yb.x, xb.y, yb.y);
        }
    } else {
        for (; k + stride < Q; k += 2 * stride) {
            const u64 k2 = k + stride;
            const u64 a0 = __ldcs(A + k), a1 = __ldcs(A + k + Q), a2 = __ldcs(A + k + 2 * Q), a3 = __ldcs(A + k + 3 * Q);
            const u64 b0 = __ldcs(B + k), b1 = __ldcs(B + k + Q), b2 = __ldcs(B + k + 2 * Q), b3 = __ldcs(B + k + 3 * Q);
            const u64 c0 = __ldcs(A + k2), c1 = __ldcs(A + k2 + Q), c2 = __ldcs(A + k2 + 2 * Q), c3 = __ldcs(A + k2 + 3 * Q);
            const u64 e0 = __ldcs(B + k2), e1 = __ldcs(B + k2 + Q), e2 = __ldcs(B + k2 + 2 * Q), e3 = __ldcs(B + k2 + 3 * Q);
            ip01_quad(s, a0, a1, a2, a3, b0, b1, b2, b3);
            ip01_quad(s, c0, c1, c2, c3, e0, e1, e2, e3);
        }
        if (k < Q) ip01_quad(s, A[k], A[k + Q], A[k + 2 * Q], A[k + 3 * Q], B[k], B[k + Q], B[k + 2 * Q], B[k + 3 * Q]);
    }
    F3 raw[3];
    raw[0] = f3_make(acc_reduce(s[0]), acc_reduce(s[1]), acc_reduce(s[2]));
    raw[1] = f3_make(acc_reduce(s[3]), acc_reduce(s[4]), acc_reduce(s[5]));
    raw[2] = f3_make(acc_reduce(s[6]), acc_reduce(s[7]), 0);
    reduce_and_finalize_seg<3>(raw, a, POL_IP01, nb, bid);
}

// Pass 2: octets x[m + jO], O = L/8, j = 0..7, of each base table.  Folding
// (x0, x4) and (x2, x6) with r0 and the results with r1 gives
//   x0 + r0 (x4 - x0) + r1 (x2 - x0) + r0 r1 (x6 - x4 - x2 + x0),
// entry m of the length-L/4 table: three base differences times the Fp3
// constants r0, r1, r0 r1, accumulated unreduced (9 products, 3 reductions).
// (x1, x5, x3, x7) give entry m + O likewise; then round 2's pair.
__device__ __forceinline__ F3 fold2(u64 x0, u64 x2, u64 x4, u64 x6, const F3& r0, const F3& r1, const F3& r01) {
    const u64 d1 = gl_sub(x4, x0), d2 = gl_sub(x2, x0), d3 = gl_sub(gl_sub(x6, x4), d2);
    AccF<FOLD_FORM> c0, c1, c2;
    c0.from(x0);
    c1.zero();
    c2.zero();
    c0.mac(d1, r0.c0); c0.mac(d2, r1.c0); c0.mac(d3, r01.c0);
    c1.mac(d1, r0.c1); c1.mac(d2, r1.c1); c1.mac(d3, r01.c1);
    c2.mac(d1, r0.c2); c2.mac(d2, r1.c2); c2.mac(d3, r01.c2);
    return f3_make(c0.reduce(), c1.reduce(), c2.reduce());
}

// LSB: octet m is entries 8m .. 8m+7; entries 2m and 2m+1 of the length-L/4
// table are fold2(y0, y2, y1, y3) and fold2(y4, y6, y5, y7).
template <bool LSB>
__device__ __forceinline__ void ip2x_body(const RoundArgs& a, u32 bid, u32 nb) {
    using P = Policy<POL_IP, 3>;
    P acc;
    acc.init();
    const F3 r0 = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    const F3 r1 = f3_make(a.chal2_ptr[0], a.chal2_ptr[1], a.chal2_ptr[2]);
    const F3 r01 = f3_mul<true, true>(r0, r1);
    const u64 O = a.L >> 3;
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    F3 lo[2], hi[2];
    for (u64 m = tid; m < O; m += stride) {
        u64 x[2][8];
#pragma unroll
        for (int t = 0; t < 2; t++) {
            if (LSB) {
                const ulonglong2* X2 = (const ulonglong2*)a.t[t].in[0] + 4 * m;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const ulonglong2 v = __ldcs(X2 + j);
                    x[t][2 * j] = v.x;
                    x[t][2 * j + 1] = v.y;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++) x[t][j] = __ldcs(a.t[t].in[0] + m + j * O);
            }
        }
#pragma unroll
        for (int t = 0; t < 2; t++) {
            if (LSB) {
                lo[t] = fold2(x[t][0], x[t][2], x[t][1], x[t][3], r0, r1, r01);
                hi[t] = fold2(x[t][4], x[t][6], x[t][5], x[t][7], r0, r1, r01);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const u64 l = c == 0 ? lo[t].c0 : c == 1 ? lo[t].c1 : lo[t].c2;
                    const u64 h = c == 0 ? hi[t].c0 : c == 1 ? hi[t].c1 : hi[t].c2;
                    ((ulonglong2*)a.t[t].out[c])[m] = make_ulonglong2(l, h);
                }
            } else {
                lo[t] = fold2(x[t][0], x[t][2], x[t][4], x[t][6], r0, r1, r01);
                hi[t] = fold2(x[t][1], x[t][3], x[t][5], x[t][7], r0, r1, r01);
                st<true>(a.t[t].out, m, lo[t]);
                st<true>(a.t[t].out, m + O, hi[t]);
            }
        }
        acc.pair(lo, hi);
    }
    F3 raw[2];
    acc.result(raw);
    reduce_and_finalize_seg<2>(raw, a, POL_IP, nb, bid);
}

}  // namespace effsc
