// k_gkr.cu -- GkrProver rounds (src/provers/gkr.rs:105-190).
//
// The reference expands the witness into two broadcast tables of 2^(2k)
// entries, w_b[b n + c] = W(b) and w_c[b n + c] = W(c), and folds all four
// tables every round.  Folding w_c over a b variable leaves it unchanged and
// folding w_b over a c variable likewise, so here the witness stays two
// compact tables: W_b (folded during the first k rounds) and W_c (folded
// during the last k); entry i of the current gate tables reads
//   W_b[i >> kc] and W_c[i & (2^kc - 1)],  kc = min(k, log2 |add|),
// the same values the broadcast tables hold.  Each round pairs (i, i + half)
// -- optionally right after folding add and mult with the previous challenge
// in the same pass.  The two ends of a pair differ in one variable: a b
// variable while the pair's W_b indices differ (the first k rounds), else a c
// variable, and the other witness table reads one entry s at both ends.  So
//   f(x) = add (W_b + W_c) + mult W_b W_c
// is quadratic in x, and the wire the reference derives from q(0), q(1), q(2),
// [q(0), (q(0) + q(2) - 2 q(1)) / 2], is q(0) and f's x^2 coefficient
//   c2 = sum d_w (d_add + d_mult s),
// d_* the differences across the pair and d_w that of the varying witness
// table: one product per pair in place of the points x = 1 and x = 2.  With
// two accumulators every fused variant fits 128 registers without spills and
// all run two blocks per SM (measured, k = 12 over Fp3: 0.98 -> 0.90 ms per
// proof; the evaluate-only variant with every table in Fp3, used on tables of
// at most two entries, spills 8 bytes).
#include "ml01.cuh"

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

// Pair (i, i + H) of the gate tables (add al / ah, mult ml / mh): q(0) gets
// the point x = 0 and c2 the product d_w (d_add + d_mult s).
template <bool EA, bool EWB, bool EWC>
__device__ __forceinline__ void gkr_pair(ProdAcc<EA, EWB || EWC>& q0, ProdAcc<EA || EWB || EWC, EWB || EWC>& qc,
                                         const RoundArgs& a, const F3& al, const F3& ah, const F3& ml, const F3& mh,
                                         u64 i, u64 H, u32 kc, u64 cm, bool bvar) {
    const F3 wbl = ld<EWB>(a.t[2].in, i >> kc), wcl = ld<EWC>(a.t[3].in, i & cm);
    gkr_point<EA, EWB, EWC>(q0, al, ml, wbl, wcl);
    const F3 da = f3_sub<EA>(ah, al), dm = f3_sub<EA>(mh, ml);
    if (bvar) {
        const F3 dw = f3_sub<EWB>(ld<EWB>(a.t[2].in, (i + H) >> kc), wbl);
        qc.mac(f3_add_mixed<EA || EWC, EA>(f3_mul<EA, EWC>(dm, wcl), da), dw);
    } else {
        const F3 dw = f3_sub<EWC>(ld<EWC>(a.t[3].in, (i + H) & cm), wcl);
        qc.mac(f3_add_mixed<EA || EWB, EA>(f3_mul<EA, EWB>(dm, wbl), da), dw);
    }
}

__device__ __forceinline__ u64 f3c(const F3& v, int c) { return c == 0 ? v.c0 : c == 1 ? v.c1 : v.c2; }

// Pairs (or quadruples) per lane of a run: a warp's run is 32 gr consecutive
// units inside one W_b index (2^kc of them), and every warp of the grid gets
// at least one.  A power of two up to 8, or 0 when a lane would get a single
// unit (the per-pair forms cost the same there).
__device__ __forceinline__ u32 gkr_run_len(u64 count, u32 kc) {
    const u64 nw = ((u64)gridDim.x * TPB) >> 5, cap = (1ULL << kc) >> 5;
    u64 g = count / (32 * nw);
    if (g > 8) g = 8;
    if (g > cap) g = cap;
    return g < 2 ? 0u : 1u << (63 - __clzll(g));
}

// Per-pair evaluation: gates(i, al, ah, ml, mh) gives the pair's gate values.
template <bool EA, bool EWB, bool EWC, class Gates>
__device__ __forceinline__ void gkr_pairs(const RoundArgs& a, u64 H, u32 kc, u64 cm, bool bvar, F3 (&raw)[2], Gates gates) {
    constexpr bool EW = EWB || EWC;
    ProdAcc<EA, EW> q0;
    ProdAcc<EA || EW, EW> qc;
    q0.init();
    qc.init();
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    for (u64 i = tid; i < H; i += stride) {
        F3 al, ah, ml, mh;
        gates(i, al, ah, ml, mh);
        gkr_pair<EA, EWB, EWC>(q0, qc, a, al, ah, ml, mh, i, H, kc, cm, bvar);
    }
    raw[0] = q0.result();
    raw[1] = qc.result();
}

// A b variable with W_c in the base field, by runs: W_b reads one entry per
// run (wl at i, wh at i + H), so a pair only accumulates add + mult s,
// add s and d_add + d_mult s (s = W_c's entry), and the run finishes
//   q(0) += wl sum (add + mult s) + sum add s,   c2 += (wh - wl) sum (d_add + d_mult s).
template <bool EA, bool EWB, class Gates>
__device__ __forceinline__ void gkr_runs(const RoundArgs& a, u64 H, u32 kc, u64 cm, u32 gr, F3 (&raw)[2], Gates gates) {
    constexpr int NC = EA ? 3 : 1;
    const u32 lane = threadIdx.x & 31;
    const u64 nw = ((u64)gridDim.x * TPB) >> 5, rl = 32ULL * gr, nruns = H / rl;
    const u64* WC = a.t[3].in[0];
    F3 q0 = f3_zero(), qc = f3_zero();
    for (u64 u = ((u64)blockIdx.x * TPB + threadIdx.x) >> 5; u < nruns; u += nw) {
        const u64 i0 = u * rl;
        Acc xa[NC], ya[NC], zd[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) xa[c] = ya[c] = zd[c] = acc_zero();
        for (u32 t = 0; t < gr; t++) {
            const u64 i = i0 + lane + 32 * t;
            F3 al, ah, ml, mh;
            gates(i, al, ah, ml, mh);
            const u64 sv = WC[i & cm];
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const u64 l = f3c(al, c);
                acc_add64(xa[c], l);
                acc_mac(xa[c], f3c(ml, c), sv);
                acc_mac(ya[c], l, sv);
                acc_add64(zd[c], gl_sub(f3c(ah, c), l));
                acc_mac(zd[c], gl_sub(f3c(mh, c), f3c(ml, c)), sv);
            }
        }
        F3 x = f3_zero(), y = f3_zero(), z = f3_zero();
        x.c0 = acc_reduce(xa[0]); y.c0 = acc_reduce(ya[0]); z.c0 = acc_reduce(zd[0]);
        if constexpr (EA) {
            x.c1 = acc_reduce(xa[1]); x.c2 = acc_reduce(xa[2]);
            y.c1 = acc_reduce(ya[1]); y.c2 = acc_reduce(ya[2]);
            z.c1 = acc_reduce(zd[1]); z.c2 = acc_reduce(zd[2]);
        }
        const F3 wl = ld<EWB>(a.t[2].in, i0 >> kc), wh = ld<EWB>(a.t[2].in, (i0 + H) >> kc);
        q0 = f3_add<true>(q0, f3_add<true>(f3_mul<EA, EWB>(x, wl), y));
        qc = f3_add<true>(qc, f3_mul<EA, EWB>(z, f3_sub<EWB>(wh, wl)));
    }
    raw[0] = q0;
    raw[1] = qc;
}

template <bool FUSED, bool EAI, bool EWB, bool EWC, bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_gkr(RoundArgs a) {
    constexpr bool EA = FUSED ? (EAI || ECH) : EAI;   // add / mult after the fold
    const u64 L = a.L;
    const u64 Ln = FUSED ? L >> 1 : L;                 // length evaluated
    const u32 lg = 63 - __clzll(Ln > 0 ? Ln : 1);
    const u32 kc = a.m_shift < lg ? a.m_shift : lg;
    const u64 cm = (1ULL << kc) - 1;
    const bool bvar = kc < lg;                         // the pairs differ in W_b's index
    F3 raw[2];
    if (Ln == 1) {
        // q(1) = 0 and q(2) = -q(0), so the wire's q(inf) is 0 (src/provers/gkr.rs:119-127)
        ProdAcc<EA, EWB || EWC> q0;
        q0.init();
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const F3 al = ld<EA>(FUSED ? (const u64* const*)a.t[0].out : a.t[0].in, 0);
            const F3 ml = ld<EA>(FUSED ? (const u64* const*)a.t[1].out : a.t[1].in, 0);
            const F3 wb = ld<EWB>(a.t[2].in, 0), wc = ld<EWC>(a.t[3].in, 0);
            gkr_point<EA, EWB, EWC>(q0, al, ml, wb, wc);
        }
        raw[0] = q0.result();
        raw[1] = f3_zero();
    } else {
        F3 rr;
        Mul3 r = load_challenge_mul(a, rr);
        if (!ECH) r = mul3_prepare<false>(rr);
        const u64 H = Ln >> 1;
        auto gates = [&](u64 i, F3& al, F3& ah, F3& ml, F3& mh) {
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
        };
        if constexpr (!EWC) {
            const u32 gr = bvar ? gkr_run_len(H, kc) : 0;
            if (gr) gkr_runs<EA, EWB>(a, H, kc, cm, gr, raw, gates);
            else gkr_pairs<EA, EWB, EWC>(a, H, kc, cm, bvar, raw, gates);
        } else {
            gkr_pairs<EA, EWB, EWC>(a, H, kc, cm, bvar, raw, gates);
        }
    }
    reduce_and_finalize<2>(raw, a, POL_GKR);
}

// Two-pass start (k >= 3, base add, mult and witness, Fp or Fp3
// challenges): rounds 0 and 1 from one pass, round 2 with a double fold from
// a second -- the GKR counterpart of ip01.cuh.
//
// Pass 1, quadruple j < Q = N/4 (N = n^2 = |add|): x_s = x[j + s Q] of add (a)
// and mult (m), the witness entries w_s = W_b[(j >> k) + s n/4] (quarter s's
// b index) and c = W_c[j mod n].  Rounds 0 and 1 both bind b variables; with
// d_s = x_{s+2} - x_s (s = 0, 1) round 0's pairs give
//   P_s = a_s (w_s + c) + c m_s w_s,  D_s = dw_s (da_s + c dm_s),
// its wire is [sum P_0 + P_1, sum D_0 + D_1], and round 1's, on the tables
// folded with r0, is quadratic in r0:
//   q(0) = sum P_0 + r0 sum B + r0^2 sum D_0,
//   B = a_0 dw_0 + da_0 (w_0 + c) + c (m_0 dw_0 + dm_0 w_0),
//   c2 = sum e g + r0 sum (f g + e h) + r0^2 sum f h,
//   e = w_1 - w_0, f = dw_1 - dw_0, g = (a_1 - a_0) + c (m_1 - m_0),
//   h = (da_1 - da_0) + c (dm_1 - dm_0).
// The eight sums take the places of POL_IP01's (T0, T1, T2, U0, U1, U2, V0,
// V2), whose finalize runs both transcript steps.
__device__ __forceinline__ void gkr01_quad(Acc (&s)[8], u64 a0, u64 a1, u64 a2, u64 a3, u64 m0, u64 m1, u64 m2, u64 m3,
                                           u64 w0, u64 w1, u64 w2, u64 w3, u64 c) {
    const u64 da0 = gl_sub(a2, a0), da1 = gl_sub(a3, a1), dm0 = gl_sub(m2, m0), dm1 = gl_sub(m3, m1);
    const u64 dw0 = gl_sub(w2, w0), dw1 = gl_sub(w3, w1);
    const u64 w0c = gl_add(w0, c);
    const u64 cdm0 = gl_mul(c, dm0), cdm1 = gl_mul(c, dm1);
    acc_mac(s[0], a0, w0c);                              // P_0
    acc_mac(s[0], c, gl_mul(m0, w0));
    acc_mac(s[6], a1, gl_add(w1, c));                    // P_1
    acc_mac(s[6], c, gl_mul(m1, w1));
    acc_mac(s[2], dw0, gl_add(da0, cdm0));               // D_0
    acc_mac(s[7], dw1, gl_add(da1, cdm1));               // D_1
    Acc t = acc_zero();                                   // B
    acc_mac(t, m0, dw0);
    acc_mac(t, dm0, w0);
    acc_mac(s[1], c, acc_reduce(t));
    acc_mac(s[1], a0, dw0);
    acc_mac(s[1], da0, w0c);
    const u64 e = gl_sub(w1, w0), f = gl_sub(dw1, dw0);
    const u64 g = gl_add(gl_sub(a1, a0), gl_mul(c, gl_sub(m1, m0)));
    const u64 h = gl_add(gl_sub(da1, da0), gl_sub(cdm1, cdm0));
    acc_mac(s[3], e, g);
    acc_mac(s[4], f, g);
    acc_mac(s[4], e, h);
    acc_mac(s[5], f, h);
}

// Runs of 32 gr quadruples inside one b (n >= 64): w_0 .. w_3 are the same
// for the whole run, so the eight sums factor into the run sums
//   X_s = sum (a_s + c m_s) (s < 4),  C_s = sum c a_s (s < 3),
// finished with the w's once per run:
//   P_0 = w_0 X_0 + C_0,  P_1 = w_1 X_1 + C_1,
//   D_0 = dw_0 (X_2 - X_0),  D_1 = dw_1 (X_3 - X_1),
//   B = dw_0 X_0 + w_0 (X_2 - X_0) + C_2 - C_0,
//   g = X_1 - X_0,  h = (X_3 - X_1) - (X_2 - X_0).
__device__ __forceinline__ void gkr01_run(Acc (&s)[8], const Acc (&x)[4], const Acc (&ca)[3], u64 w0, u64 w1, u64 w2,
                                          u64 w3) {
    const u64 X0 = acc_reduce(x[0]), X1 = acc_reduce(x[1]), X2 = acc_reduce(x[2]), X3 = acc_reduce(x[3]);
    const u64 C0 = acc_reduce(ca[0]), C1 = acc_reduce(ca[1]), C2 = acc_reduce(ca[2]);
    const u64 dw0 = gl_sub(w2, w0), dw1 = gl_sub(w3, w1), e = gl_sub(w1, w0), f = gl_sub(dw1, dw0);
    const u64 d20 = gl_sub(X2, X0), d31 = gl_sub(X3, X1), g = gl_sub(X1, X0), h = gl_sub(d31, d20);
    acc_mac(s[0], w0, X0);
    acc_add64(s[0], C0);
    acc_mac(s[6], w1, X1);
    acc_add64(s[6], C1);
    acc_mac(s[2], dw0, d20);
    acc_mac(s[7], dw1, d31);
    acc_mac(s[1], dw0, X0);
    acc_mac(s[1], w0, d20);
    acc_add64(s[1], gl_sub(C2, C0));
    acc_mac(s[3], e, g);
    acc_mac(s[4], f, g);
    acc_mac(s[4], e, h);
    acc_mac(s[5], f, h);
}

__global__ void __launch_bounds__(TPB, 2) k_gkr_r01(RoundArgs a) {
    Acc s[8];
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = acc_zero();
    const u64 Q = a.L >> 2;
    const u32 k = a.m_shift;
    const u64 nq = (1ULL << k) >> 2, cm = (1ULL << k) - 1;
    const u64* A = a.t[0].in[0];
    const u64* M = a.t[1].in[0];
    const u64* WB = a.t[2].in[0];
    const u64* WC = a.t[3].in[0];
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    for (u64 j = tid; j < Q; j += stride) {
        const u64 a0 = __ldcs(A + j), a1 = __ldcs(A + j + Q), a2 = __ldcs(A + j + 2 * Q), a3 = __ldcs(A + j + 3 * Q);
        const u64 m0 = __ldcs(M + j), m1 = __ldcs(M + j + Q), m2 = __ldcs(M + j + 2 * Q), m3 = __ldcs(M + j + 3 * Q);
        const u64 b = j >> k;
        gkr01_quad(s, a0, a1, a2, a3, m0, m1, m2, m3, WB[b], WB[b + nq], WB[b + 2 * nq], WB[b + 3 * nq], WC[j & cm]);
    }
    F3 raw[3];
    raw[0] = f3_make(acc_reduce(s[0]), acc_reduce(s[1]), acc_reduce(s[2]));
    raw[1] = f3_make(acc_reduce(s[3]), acc_reduce(s[4]), acc_reduce(s[5]));
    raw[2] = f3_make(acc_reduce(s[6]), acc_reduce(s[7]), 0);
    reduce_and_finalize_seg<3>(raw, a, POL_IP01, gridDim.x, blockIdx.x);
}

// Pass 1 by runs, for large tables: a warp takes 32 gr consecutive
// quadruples inside one b (gkr01_run's factored sums, two quadruples per
// iteration so that sixteen loads are in flight), and each lane keeps its
// eight sums reduced in shared memory (updated once per run with the run's
// w's) instead of in registers: 80 registers, three blocks per SM (measured,
// k = 12: 102 -> 85 us for the pass, 0.777 -> 0.757 ms per proof).  gr is a
// power of two from 2 to 16; the host launches this kernel only when every
// warp gets a run of at least two quadruples per lane.
__global__ void __launch_bounds__(TPB, 3) k_gkr_r01_runs(RoundArgs a) {
    __shared__ u64 s_sum[8][TPB];
    for (int t = 0; t < 8; t++) s_sum[t][threadIdx.x] = 0;
    const u64 Q = a.L >> 2;
    const u32 k = a.m_shift;
    const u64 nq = (1ULL << k) >> 2, cm = (1ULL << k) - 1;
    const u64* A = a.t[0].in[0];
    const u64* M = a.t[1].in[0];
    const u64* WB = a.t[2].in[0];
    const u64* WC = a.t[3].in[0];
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    const u64 nw = stride >> 5, capk = (1ULL << k) >> 5;
    u64 g = Q / (32 * nw);
    if (g > 16) g = 16;
    if (g > capk) g = capk;
    const u32 gr = g < 2 ? 2u : 1u << (63 - __clzll(g));   // the host launches this kernel only when g >= 2
    const u32 lane = threadIdx.x & 31;
    const u64 rl = 32ULL * gr, nruns = Q / rl;
    for (u64 u = tid >> 5; u < nruns; u += nw) {
        const u64 i0 = u * rl;
        Acc x[4], ca[3];
#pragma unroll
        for (int t = 0; t < 4; t++) x[t] = acc_zero();
#pragma unroll
        for (int t = 0; t < 3; t++) ca[t] = acc_zero();
        for (u32 t = 0; t < gr; t += 2) {
            u64 av[2][4], mv[2][4], c[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const u64 j = i0 + lane + 32 * (t + h);
#pragma unroll
                for (int q = 0; q < 4; q++) { av[h][q] = __ldcs(A + j + q * Q); mv[h][q] = __ldcs(M + j + q * Q); }
                c[h] = WC[j & cm];
            }
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    acc_add64(x[q], av[h][q]);
                    acc_mac(x[q], c[h], mv[h][q]);
                    if (q < 3) acc_mac(ca[q], c[h], av[h][q]);
                }
        }
        const u64 b = i0 >> k;
        Acc d[8];
#pragma unroll
        for (int t = 0; t < 8; t++) d[t] = acc_from(s_sum[t][threadIdx.x]);
        gkr01_run(d, x, ca, WB[b], WB[b + nq], WB[b + 2 * nq], WB[b + 3 * nq]);
#pragma unroll
        for (int t = 0; t < 8; t++) s_sum[t][threadIdx.x] = acc_reduce(d[t]);
    }
    F3 raw[3];
    raw[0] = f3_make(s_sum[0][threadIdx.x], s_sum[1][threadIdx.x], s_sum[2][threadIdx.x]);
    raw[1] = f3_make(s_sum[3][threadIdx.x], s_sum[4][threadIdx.x], s_sum[5][threadIdx.x]);
    raw[2] = f3_make(s_sum[6][threadIdx.x], s_sum[7][threadIdx.x], 0);
    reduce_and_finalize_seg<3>(raw, a, POL_IP01, gridDim.x, blockIdx.x);
}

// Pass 2: add and mult folded with r0 and r1 at once from the base tables
// (ml_fold2 on the quarters x[i + s Q]; the entry i + H of the length-Q table
// from x[i + H + s Q], H = Q/2), written out, and round 2 -- a b variable,
// k >= 3 -- evaluated on them with W_b folded twice (t[2]) and W_c as is.
template <bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_gkr_r2x(RoundArgs a) {
    constexpr bool EA = ECH, EWB = ECH;
    const F3 r0 = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    const F3 r1 = f3_make(a.chal2_ptr[0], a.chal2_ptr[1], a.chal2_ptr[2]);
    const F3 r01 = f3_mul<ECH, ECH>(r0, r1);
    const u64 Q = a.L >> 2, H = Q >> 1;
    const u32 kc = a.m_shift;
    const u64 cm = (1ULL << kc) - 1;
    auto gates = [&](u64 i, F3& al, F3& ah, F3& ml, F3& mh) {
        F3 lo[2], hi[2];
#pragma unroll
        for (int t = 0; t < 2; t++) {
            const u64* X = a.t[t].in[0];
            u64 x[8];
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = __ldcs(X + i + j * H);
            lo[t] = ml_fold2<ECH>(x[0], x[2], x[4], x[6], r0, r1, r01);
            hi[t] = ml_fold2<ECH>(x[1], x[3], x[5], x[7], r0, r1, r01);
            st<EA>(a.t[t].out, i, lo[t]);
            st<EA>(a.t[t].out, i + H, hi[t]);
        }
        al = lo[0]; ah = hi[0]; ml = lo[1]; mh = hi[1];
    };
    F3 raw[2];
    const u32 gr = gkr_run_len(H, kc);
    if (gr) gkr_runs<EA, EWB>(a, H, kc, cm, gr, raw, gates);
    else gkr_pairs<EA, EWB, false>(a, H, kc, cm, true, raw, gates);
    reduce_and_finalize_seg<2>(raw, a, POL_GKR, gridDim.x, blockIdx.x);
}

bool launch_gkr01(const RoundArgs& a, int grid, cudaStream_t s) {
    k_gkr_r01<<<grid, TPB, 0, s>>>(a);
    return true;
}
bool launch_gkr01_runs(const RoundArgs& a, int grid, cudaStream_t s) {
    k_gkr_r01_runs<<<grid, TPB, 0, s>>>(a);
    return true;
}
bool launch_gkr2x(bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    if (ech) k_gkr_r2x<true><<<grid, TPB, 0, s>>>(a);
    else k_gkr_r2x<false><<<grid, TPB, 0, s>>>(a);
    return true;
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
