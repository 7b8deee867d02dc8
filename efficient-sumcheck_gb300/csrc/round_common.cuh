// round_common.cuh -- building blocks of the sumcheck round kernels.
//
// One round of every prover is a single pass over its tables:
//   fold with the previous challenge (new = lo + (hi - lo) * r) and accumulate
//   the next round polynomial, each element read once and written once.
// Per-thread sums are kept unreduced (gl.cuh Acc), reduced once per thread,
// combined across the warp with shuffles, across the block in shared memory,
// and across the grid by the last block to finish (atomic ticket), which also
// turns the raw sums into the EvalsInfty wire values (reference
// src/sumcheck_prover.rs:40-59) and, on the device-resident path, runs the
// transcript step: absorb the wire values and the hook bytes, squeeze the
// next challenge (reference src/runner.rs:39-55).
#pragma once
#include "gl.cuh"
#include "keccak.cuh"
#include "kernels.h"

namespace effsc {

constexpr int TPB = KERNEL_TPB;
constexpr int NWARP = TPB / 32;
constexpr int RAW_WORDS = 12;   // up to 4 Fp3 raw values per block partial

template <u32 M>
__device__ __forceinline__ constexpr bool ext_of(int t) { return (M >> t) & 1u; }

// Start of every kernel launched by launch_chain: wait until the previous
// kernel on the stream has completed and its writes are visible, then let the
// next kernel be scheduled (it waits the same way before it reads anything).
__device__ __forceinline__ void chain_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <bool E>
__device__ __forceinline__ F3 ld(const u64* const* p, u64 i) {
    F3 r;
    r.c0 = p[0][i];
    if (E) { r.c1 = p[1][i]; r.c2 = p[2][i]; } else { r.c1 = r.c2 = 0; }
    return r;
}
template <bool E>
__device__ __forceinline__ void st(u64* const* p, u64 i, const F3& v) {
    p[0][i] = v.c0;
    if (E) { p[1][i] = v.c1; p[2][i] = v.c2; }
}
// Table t of a kernel whose ext mask is M (t is a compile-time constant after
// unrolling, so the branch folds away).
template <u32 M>
__device__ __forceinline__ F3 ldm(const u64* const* p, u64 i, int t) {
    return ((M >> t) & 1u) ? ld<true>(p, i) : ld<false>(p, i);
}
__device__ __forceinline__ u64 next_pow2_dev(u64 n) {
    return n <= 1 ? 1 : (1ULL << (64 - __clzll(n - 1)));
}

// ---------------------------------------------------------------------------
// Policies: what a round accumulates for each (lo, hi) pair of table entries.
//   pair(lo, hi): a regular pair
//   tail(lo)    : MSB tail entry whose hi is an implicit zero
//   single(lo)  : an entry with no partner that only feeds h(0) (LSB remainder,
//                 and the length-1 case)
// ---------------------------------------------------------------------------
template <int POL, u32 M>
struct Policy;

// MultilinearProver: s0 = sum lo, s1 = sum hi (src/multilinear_sumcheck.rs:86-124,
// src/provers/multilinear_lsb.rs:60-96).
template <u32 M>
struct Policy<POL_ML, M> {
    static constexpr int NT = 1, NRAW = 2;
    static constexpr bool LSB_REMAINDER = true;
    static constexpr bool E0 = ext_of<M>(0);
    SumAcc<E0> s0, s1;
    __device__ __forceinline__ void init() { s0.init(); s1.init(); }
    __device__ __forceinline__ void pair(const F3* lo, const F3* hi) { s0.add(lo[0]); s1.add(hi[0]); }
    __device__ __forceinline__ void tail(const F3* lo) { s0.add(lo[0]); }
    __device__ __forceinline__ void single(const F3* lo) { s0.add(lo[0]); }
    __device__ __forceinline__ void result(F3* o) const { o[0] = s0.result(); o[1] = s1.result(); }
};

// InnerProductProver: q0 = sum a_lo b_lo, qinf = sum (a_hi - a_lo)(b_hi - b_lo);
// MSB tail adds a*b to both (src/provers/inner_product.rs:94-110), the LSB
// remainder to q0 only (src/provers/inner_product_lsb.rs:131-139).
template <u32 M>
struct IpLike {
    static constexpr int NT = 2, NRAW = 2;
    static constexpr bool LSB_REMAINDER = true;
    static constexpr bool E0 = ext_of<M>(0), E1 = ext_of<M>(1);
    ProdAcc<E0, E1> q0, qi;
    __device__ __forceinline__ void init() { q0.init(); qi.init(); }
    __device__ __forceinline__ void pair(const F3* lo, const F3* hi) {
        q0.mac(lo[0], lo[1]);
        qi.mac(f3_sub<E0>(hi[0], lo[0]), f3_sub<E1>(hi[1], lo[1]));
    }
    __device__ __forceinline__ void tail(const F3* lo) { q0.mac(lo[0], lo[1]); qi.mac(lo[0], lo[1]); }
    __device__ __forceinline__ void single(const F3* lo) { q0.mac(lo[0], lo[1]); }
    __device__ __forceinline__ void result(F3* o) const { o[0] = q0.result(); o[1] = qi.result(); }
};
template <u32 M> struct Policy<POL_IP, M> : IpLike<M> {};
// EqFactored right phase (src/provers/eq_factored.rs:178-209): tables (eq_r, p).
template <u32 M> struct Policy<POL_EQFR, M> : IpLike<M> {};

// CoefficientProver with the product evaluator: coefficients of
// prod_i (lo_i + x (hi_i - lo_i)).  k = 1 is Degree1Eval
// (src/provers/coefficient.rs:341-351), k = 3 is TripleProductEval
// (tests/adversarial_verifier.rs:444-466).  No tails: the coefficient provers
// fold with floor(L/2) (src/provers/coefficient.rs:131-140).
template <u32 M>
struct Policy<POL_C1, M> {
    static constexpr int NT = 1, NRAW = 2;
    static constexpr bool LSB_REMAINDER = false;
    static constexpr bool E0 = ext_of<M>(0);
    SumAcc<E0> c0, c1;
    __device__ __forceinline__ void init() { c0.init(); c1.init(); }
    __device__ __forceinline__ void pair(const F3* lo, const F3* hi) {
        c0.add(lo[0]);
        c1.add(f3_sub<E0>(hi[0], lo[0]));
    }
    __device__ __forceinline__ void tail(const F3*) {}
    __device__ __forceinline__ void single(const F3*) {}
    __device__ __forceinline__ void result(F3* o) const { o[0] = c0.result(); o[1] = c1.result(); }
};
template <u32 M>
struct Policy<POL_C2, M> {
    static constexpr int NT = 2, NRAW = 3;
    static constexpr bool LSB_REMAINDER = false;
    static constexpr bool E0 = ext_of<M>(0), E1 = ext_of<M>(1);
    ProdAcc<E0, E1> c0, c1, c2;
    __device__ __forceinline__ void init() { c0.init(); c1.init(); c2.init(); }
    __device__ __forceinline__ void pair(const F3* lo, const F3* hi) {
        F3 da = f3_sub<E0>(hi[0], lo[0]), db = f3_sub<E1>(hi[1], lo[1]);
        c0.mac(lo[0], lo[1]);
        c1.mac(lo[0], db);
        c1.mac(da, lo[1]);
        c2.mac(da, db);
    }
    __device__ __forceinline__ void tail(const F3*) {}
    __device__ __forceinline__ void single(const F3*) {}
    __device__ __forceinline__ void result(F3* o) const { o[0] = c0.result(); o[1] = c1.result(); o[2] = c2.result(); }
};
// Degree 3 (TripleProductEval, eq * f * g) by point values: h(x) = A(x) B(x)
// C(x) at x = 0, 1, 2 and the leading coefficient (x = inf), 18 products per
// point with the first product reduced (72 per pair instead of 90 for the
// four coefficients); the last block turns them into the wire [h(0), h(inf),
// h(2)] and the coefficients (c0, c1) of the per-round aux pair.
template <u32 M>
struct Policy<POL_C3, M> {
    static constexpr int NT = 3, NRAW = 4;
    static constexpr bool LSB_REMAINDER = false;
    static constexpr bool E0 = ext_of<M>(0), E1 = ext_of<M>(1), E2 = ext_of<M>(2);
    static constexpr bool EU = E0 || E1;
    PointAcc<EU, E2> h0, h1, h2, hi;
    __device__ __forceinline__ void init() { h0.init(); h1.init(); h2.init(); hi.init(); }
    __device__ __forceinline__ void point(PointAcc<EU, E2>& acc, const F3& a, const F3& b, const F3& c) {
        acc.mac(f3_mul<E0, E1>(a, b), c);
    }
    __device__ __forceinline__ void pair(const F3* lo, const F3* hi_) {
        const F3 da = f3_sub<E0>(hi_[0], lo[0]), db = f3_sub<E1>(hi_[1], lo[1]), dc = f3_sub<E2>(hi_[2], lo[2]);
        point(h0, lo[0], lo[1], lo[2]);
        point(h1, hi_[0], hi_[1], hi_[2]);
        point(h2, f3_add<E0>(hi_[0], da), f3_add<E1>(hi_[1], db), f3_add<E2>(hi_[2], dc));
        point(hi, da, db, dc);
    }
    __device__ __forceinline__ void tail(const F3*) {}
    __device__ __forceinline__ void single(const F3*) {}
    __device__ __forceinline__ void result(F3* o) const {
        o[0] = h0.result(); o[1] = h1.result(); o[2] = h2.result(); o[3] = hi.result();
    }
};

// The degree-3 evaluator for the device protocol: h(0), h(2) and h(inf) only
// (the wire), one accumulator and one product fewer per pair than POL_C3.
template <u32 M>
struct Policy<POL_C3W, M> {
    static constexpr int NT = 3, NRAW = 3;
    static constexpr bool LSB_REMAINDER = false;
    static constexpr bool E0 = ext_of<M>(0), E1 = ext_of<M>(1), E2 = ext_of<M>(2);
    static constexpr bool EU = E0 || E1;
    PointAcc<EU, E2> h0, h2, hi;
    __device__ __forceinline__ void init() { h0.init(); h2.init(); hi.init(); }
    __device__ __forceinline__ void point(PointAcc<EU, E2>& acc, const F3& a, const F3& b, const F3& c) {
        acc.mac(f3_mul<E0, E1>(a, b), c);
    }
    __device__ __forceinline__ void pair(const F3* lo, const F3* hi_) {
        const F3 da = f3_sub<E0>(hi_[0], lo[0]), db = f3_sub<E1>(hi_[1], lo[1]), dc = f3_sub<E2>(hi_[2], lo[2]);
        point(h0, lo[0], lo[1], lo[2]);
        point(h2, f3_add<E0>(hi_[0], da), f3_add<E1>(hi_[1], db), f3_add<E2>(hi_[2], dc));
        point(hi, da, db, dc);
    }
    __device__ __forceinline__ void tail(const F3*) {}
    __device__ __forceinline__ void single(const F3*) {}
    __device__ __forceinline__ void result(F3* o) const { o[0] = h0.result(); o[1] = h2.result(); o[2] = hi.result(); }
};

// ---------------------------------------------------------------------------
// Finalisation by the last block.
// ---------------------------------------------------------------------------
__device__ __forceinline__ F3 ld_scalar(const u64* const* p) {
    F3 r;
    r.c0 = p[0] ? p[0][0] : 0;
    r.c1 = p[1] ? p[1][0] : 0;
    r.c2 = p[2] ? p[2][0] : 0;
    return r;
}

__device__ __forceinline__ int pol_nwire_dev(int pol) {
    switch (pol) {
    case POL_ML: case POL_C1: case POL_X1: return 1;
    case POL_X2: return 2;
    case POL_X3: return 3;
    case POL_C3: case POL_C3W: return 3;
    default: return 2;
    }
}

// POL_IP01: the last block holds the eight base-field sums of one pass over
// the InnerProduct base tables (quadruples x_j = x[k + jQ], Q = L/4,
// da = x2 - x0, da' = x3 - x1):
//   T0 = sum a0 b0, T1 = sum a0 db + da b0, T2 = sum da db,
//   U0 = sum ea eb, U1 = sum ea fb + fa eb, U2 = sum fa fb
//       (ea = a1 - a0, fa = da' - da),
//   V0 = sum a1 b1, V2 = sum da' db'.
// Round 0 (src/provers/inner_product.rs:94-103): [T0 + V0, T2 + V2].
// Round 1 on the tables folded with r0 is a quadratic in r0:
//   h(0) = T0 + r0 T1 + r0^2 T2, h(inf) = U0 + r0 U1 + r0^2 U2.
// Both rounds run the transcript step in order (wire, hook, challenge).
static __device__ __noinline__ void finalize_ip01(const u64* raw, const RoundArgs& a) {
    __shared__ u64 s_w[2][6];
    __shared__ u64 s_c[2][3];
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        s_w[0][0] = gl_add(raw[0], raw[6]); s_w[0][1] = 0; s_w[0][2] = 0;
        s_w[0][3] = gl_add(raw[2], raw[7]); s_w[0][4] = 0; s_w[0][5] = 0;
    }
    __syncwarp();
    DevTranscript* T = (DevTranscript*)a.tx.tx;
    WarpTx w = tx_load(T, lane);
    for (int rd = 0; rd < 2; rd++) {
        if (rd == 1 && lane == 0) {
            const F3 r = f3_make(s_c[0][0], s_c[0][1], s_c[0][2]);
            F3 q0 = f3_make(raw[2], 0, 0), qi = f3_make(raw[5], 0, 0);
            q0 = f3_add<true>(f3_mul<true, true>(q0, r), f3_make(raw[1], 0, 0));
            q0 = f3_add<true>(f3_mul<true, true>(q0, r), f3_make(raw[0], 0, 0));
            qi = f3_add<true>(f3_mul<true, true>(qi, r), f3_make(raw[4], 0, 0));
            qi = f3_add<true>(f3_mul<true, true>(qi, r), f3_make(raw[3], 0, 0));
            s_w[1][0] = q0.c0; s_w[1][1] = q0.c1; s_w[1][2] = q0.c2;
            s_w[1][3] = qi.c0; s_w[1][4] = qi.c1; s_w[1][5] = qi.c2;
        }
        __syncwarp();
        tx_send_elems(w, lane, s_w[rd], 2);
        if (a.tx.hook_len) {
            const uint8_t* hk = a.tx.hook;
            tx_absorb(w, lane, a.tx.hook_len, [&](u32 k) -> uint8_t { return hk[k]; });
        }
        tx_challenge(w, lane, s_c[rd], s_scr);
    }
    tx_store(T, w, lane);
    if (lane < 12) a.tx.proof_wire[lane] = s_w[lane / 6][lane % 6];
    if (lane < 6) a.tx.proof_chal[lane] = s_c[lane / 3][lane % 3];
}

// POL_ML01: raw = the quarter sums (S0, S1, S2) of a Multilinear base
// table.  Round 0's wire is S0 + S1; round 1's is S0 + r0 (S2 - S0).  Both
// transcript steps (send, hook, challenge) run here.
static __device__ __noinline__ void finalize_ml01(const u64* raw, const RoundArgs& a) {
    __shared__ u64 s_w[2][3];
    __shared__ u64 s_c[2][3];
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x & 31;
    if (lane == 0) { s_w[0][0] = gl_add(raw[0], raw[1]); s_w[0][1] = 0; s_w[0][2] = 0; }
    __syncwarp();
    DevTranscript* T = (DevTranscript*)a.tx.tx;
    WarpTx w = tx_load(T, lane);
    for (int rd = 0; rd < 2; rd++) {
        if (rd == 1 && lane == 0) {
            const F3 r = f3_make(s_c[0][0], s_c[0][1], s_c[0][2]);
            const F3 v = f3_add<true>(f3_make(raw[0], 0, 0), f3_mul<true, true>(f3_make(gl_sub(raw[2], raw[0]), 0, 0), r));
            s_w[1][0] = v.c0; s_w[1][1] = v.c1; s_w[1][2] = v.c2;
        }
        __syncwarp();
        tx_send_elems(w, lane, s_w[rd], 1);
        if (a.tx.hook_len) {
            const uint8_t* hk = a.tx.hook;
            tx_absorb(w, lane, a.tx.hook_len, [&](u32 k) -> uint8_t { return hk[k]; });
        }
        tx_challenge(w, lane, s_c[rd], s_scr);
    }
    tx_store(T, w, lane);
    if (lane < 6) a.tx.proof_wire[lane] = s_w[lane / 3][lane % 3];
    if (lane < 6) a.tx.proof_chal[lane] = s_c[lane / 3][lane % 3];
}

// raw: NRAW Fp3 values in shared memory (3 words each).  Run by warp 0.
static __device__ __noinline__ void finalize_warp(int pol, const u64* raw, const RoundArgs& a) {
    if (pol == POL_IP01) {
        finalize_ip01(raw, a);
        return;
    }
    if (pol == POL_ML01) {
        finalize_ml01(raw, a);
        return;
    }
    __shared__ u64 s_wire[9];
    __shared__ u64 s_aux[6];
    __shared__ u64 s_chal[3];
    __shared__ __align__(8) uint8_t s_scratch[64];
    const int lane = threadIdx.x & 31;
    int nwire = pol_nwire_dev(pol);
    if (lane == 0) {
        F3 r[4];
        for (int i = 0; i < 4; i++) r[i] = f3_make(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]);
        F3 w[3];
        if (pol == POL_EQFR) {
            F3 sc = ld_scalar(a.scalar);
            r[0] = f3_mul<true, true>(r[0], sc);
            r[1] = f3_mul<true, true>(r[1], sc);
        }
        switch (pol) {
        case POL_ML: case POL_C1:
            w[0] = r[0];
            break;
        case POL_C2:
            w[0] = r[0]; w[1] = r[2];
            break;
        case POL_C3: {
            // r = h(0), h(1), h(2), h(inf): wire [h(0), h(inf), h(2)]; the
            // aux pair is (c0, c1) of h = c0 + c1 x + c2 x^2 + c3 x^3:
            // A = h(1) - c0 - c3 = c1 + c2, B = h(2) - c0 - 8 c3 = 2 c1 + 4 c2
            w[0] = r[0]; w[1] = r[3]; w[2] = r[2];
            const u64 inv2 = 0x7FFFFFFF80000001ULL;   // (p + 1) / 2
            const F3 c3x2 = f3_add<true>(r[3], r[3]), c3x4 = f3_add<true>(c3x2, c3x2);
            const F3 A = f3_sub<true>(f3_sub<true>(r[1], r[0]), r[3]);
            const F3 B = f3_sub<true>(f3_sub<true>(r[2], r[0]), f3_add<true>(c3x4, c3x4));
            const F3 t = f3_sub<true>(B, f3_add<true>(A, A));
            const F3 c2 = f3_make(gl_mul(t.c0, inv2), gl_mul(t.c1, inv2), gl_mul(t.c2, inv2));
            r[1] = f3_sub<true>(A, c2);
            break;
        }
        case POL_C3W:
            // r = h(0), h(2), h(inf): wire [h(0), h(inf), h(2)]; no aux pair
            w[0] = r[0]; w[1] = r[2]; w[2] = r[1];
            r[1] = f3_zero();
            break;
        case POL_X1: case POL_X2: case POL_X3: {
            // r = the coefficients c0..c3 of h; the EvalsInfty wire
            // (src/provers/coefficient.rs:272-294): [h(0)] for degree 1,
            // [h(0), h(inf)] for 2, [h(0), h(inf), h(2)] for 3; aux (c0, c1)
            w[0] = r[0];
            if (pol == POL_X2) w[1] = r[2];
            if (pol == POL_X3) {
                w[1] = r[3];
                const F3 two = f3_make(2, 0, 0);
                w[2] = f3_add<true>(f3_mul<true, true>(f3_add<true>(f3_mul<true, true>(
                    f3_add<true>(f3_mul<true, true>(r[3], two), r[2]), two), r[1]), two), r[0]);
            }
            break;
        }
        case POL_GKR:
            // r = q(0), c2: q is quadratic, so the reference's
            // q(inf) = (q(0) + q(2) - 2 q(1)) / 2 (src/provers/gkr.rs:185-189) is c2
            w[0] = r[0]; w[1] = r[1];
            break;
        default:   // IP, EQF
            w[0] = r[0]; w[1] = r[1];
            break;
        }
        for (int i = 0; i < nwire; i++) { s_wire[3 * i] = w[i].c0; s_wire[3 * i + 1] = w[i].c1; s_wire[3 * i + 2] = w[i].c2; }
        s_aux[0] = r[0].c0; s_aux[1] = r[0].c1; s_aux[2] = r[0].c2;
        s_aux[3] = r[1].c0; s_aux[4] = r[1].c1; s_aux[5] = r[1].c2;
    }
    __syncwarp();
    if (a.result) {
        for (int i = lane; i < 3 * nwire; i += 32) a.result[i] = s_wire[i];
        if (lane < 6) a.result[3 * nwire + lane] = s_aux[lane];
    }
    if (a.tx.tx) {
        DevTranscript* T = (DevTranscript*)a.tx.tx;
        WarpTx w = tx_load(T, lane);
        tx_send_elems(w, lane, s_wire, nwire);
        if (a.tx.hook_len) {
            const uint8_t* hk = a.tx.hook;
            if (((w.pos & 7) == 0 || w.squeezing) && (a.tx.hook_len & 7) == 0 && ((uintptr_t)hk & 7) == 0) {
                const u64* hw = (const u64*)hk;
                tx_absorb_words(w, lane, a.tx.hook_len >> 3, [&](u32 k) -> u64 { return hw[k]; });
            } else {
                tx_absorb(w, lane, a.tx.hook_len, [&](u32 k) -> uint8_t { return hk[k]; });
            }
        }
        tx_challenge(w, lane, s_chal, s_scratch);
        tx_store(T, w, lane);
        if (lane < 3) {
            if (a.tx.chal_next) a.tx.chal_next[lane] = s_chal[lane];
            if (a.tx.proof_chal) a.tx.proof_chal[lane] = s_chal[lane];
        }
        if (a.tx.proof_wire)
            for (int i = lane; i < 3 * nwire; i += 32) a.tx.proof_wire[i] = s_wire[i];
    }
}

// Block + grid reduction of NRAW Fp3 values over the nb blocks of one round
// (this block is number bid); the last block to finish finalises.
template <int NRAW>
__device__ __forceinline__ void reduce_and_finalize_seg(F3 (&v)[NRAW], const RoundArgs& a, int pol, u32 nb, u32 bid) {
    __shared__ u64 s_red[NWARP][RAW_WORDS];
    __shared__ u64 s_tot[RAW_WORDS];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
#pragma unroll
        for (int i = 0; i < NRAW; i++) {
            v[i].c0 = gl_add(v[i].c0, __shfl_down_sync(0xffffffffu, v[i].c0, off));
            v[i].c1 = gl_add(v[i].c1, __shfl_down_sync(0xffffffffu, v[i].c1, off));
            v[i].c2 = gl_add(v[i].c2, __shfl_down_sync(0xffffffffu, v[i].c2, off));
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NRAW; i++) { s_red[warp][3 * i] = v[i].c0; s_red[warp][3 * i + 1] = v[i].c1; s_red[warp][3 * i + 2] = v[i].c2; }
    }
    __syncthreads();
    if (threadIdx.x < 3 * NRAW) {
        u64 s = 0;
#pragma unroll
        for (int w = 0; w < NWARP; w++) s = gl_add(s, s_red[w][threadIdx.x]);
        if (nb == 1) s_tot[threadIdx.x] = s;
        else a.partials[(u64)bid * RAW_WORDS + threadIdx.x] = s;
    }
    if (nb > 1) {
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            u32 t = atomicAdd(a.counter, 1u);
            s_last = (t == nb - 1);
        }
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        // every thread owns one of the 3*NRAW words and walks the partials
        // (unrolled so that several blocks' loads are in flight at once)
        u64 acc[RAW_WORDS];
#pragma unroll
        for (int i = 0; i < 3 * NRAW; i++) acc[i] = 0;
#pragma unroll 4
        for (u32 b = threadIdx.x; b < nb; b += TPB)
#pragma unroll
            for (int i = 0; i < 3 * NRAW; i++) acc[i] = gl_add(acc[i], __ldcg(&a.partials[(u64)b * RAW_WORDS + i]));
#pragma unroll
        for (int off = 16; off; off >>= 1)
            for (int i = 0; i < 3 * NRAW; i++) acc[i] = gl_add(acc[i], __shfl_down_sync(0xffffffffu, acc[i], off));
        __syncthreads();
        if (lane == 0)
            for (int i = 0; i < 3 * NRAW; i++) s_red[warp][i] = acc[i];
        __syncthreads();
        if (threadIdx.x < 3 * NRAW) {
            u64 s = 0;
            for (int w = 0; w < NWARP; w++) s = gl_add(s, s_red[w][threadIdx.x]);
            s_tot[threadIdx.x] = s;
        }
        if (threadIdx.x == 0) *a.counter = 0;
    }
    __syncthreads();
    if (NRAW < 4 && threadIdx.x < 3 * (4 - NRAW)) s_tot[3 * NRAW + threadIdx.x] = 0;
    __syncthreads();
    if (warp == 0) finalize_warp(pol, s_tot, a);
}

template <int NRAW>
__device__ __forceinline__ void reduce_and_finalize(F3 (&v)[NRAW], const RoundArgs& a, int pol) {
    reduce_and_finalize_seg<NRAW>(v, a, pol, gridDim.x, blockIdx.x);
}

__device__ __forceinline__ Mul3 load_challenge_mul(const RoundArgs& a, F3& r) {
    if (a.chal_ptr) r = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    else r = f3_make(a.chal[0], a.chal[1], a.chal[2]);
    return mul3_prepare<true>(r);
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Unfused evaluation of the round polynomial on the current tables.
template <int POL, int SEM, u32 M>
__device__ __forceinline__ void eval_body(const RoundArgs& a, u32 bid, u32 nb) {
    using P = Policy<POL, M>;
    P acc;
    acc.init();
    const u64 L = a.L;
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    F3 lo[3], hi[3];
    if (SEM == SEM_MSB_PAD) {
        if (L == 1) {
            if (tid == 0) {
#pragma unroll
                for (int t = 0; t < P::NT; t++) lo[t] = ldm<M>(a.t[t].in, 0, t);
                acc.single(lo);
            }
        } else if (L > 1) {
            const u64 half = next_pow2_dev(L) >> 1, paired = L - half;
            for (u64 j = tid; j < half; j += stride) {
#pragma unroll
                for (int t = 0; t < P::NT; t++) lo[t] = ldm<M>(a.t[t].in, j, t);
                if (j < paired) {
#pragma unroll
                    for (int t = 0; t < P::NT; t++) hi[t] = ldm<M>(a.t[t].in, j + half, t);
                    acc.pair(lo, hi);
                } else {
                    acc.tail(lo);
                }
            }
        }
    } else if (SEM == SEM_MSB_FLOOR) {
        const u64 half = L / 2;
        for (u64 j = tid; j < half; j += stride) {
#pragma unroll
            for (int t = 0; t < P::NT; t++) {
                lo[t] = ldm<M>(a.t[t].in, j, t);
                hi[t] = ldm<M>(a.t[t].in, j + half, t);
            }
            acc.pair(lo, hi);
        }
    } else {
        const u64 n = P::LSB_REMAINDER ? (L + 1) / 2 : L / 2;
        for (u64 j = tid; j < n; j += stride) {
#pragma unroll
            for (int t = 0; t < P::NT; t++) lo[t] = ldm<M>(a.t[t].in, 2 * j, t);
            if (2 * j + 1 < L) {
#pragma unroll
                for (int t = 0; t < P::NT; t++) hi[t] = ldm<M>(a.t[t].in, 2 * j + 1, t);
                acc.pair(lo, hi);
            } else {
                acc.single(lo);
            }
        }
    }
    F3 raw[P::NRAW];
    acc.result(raw);
    reduce_and_finalize_seg<P::NRAW>(raw, a, POL, nb, bid);
}
template <int POL, int SEM, u32 M>
__global__ void __launch_bounds__(TPB) k_eval(RoundArgs a) {
    chain_enter();
    eval_body<POL, SEM, M>(a, blockIdx.x, gridDim.x);
}

// Fused fold + evaluate.  Requires L % 4 == 0 (and L a power of two for the
// padded MSB semantics): then the fold has no tail and the next round's pairs
// are exactly the quadruples (k, k+Q, k+2Q, k+3Q) (MSB) or (4k..4k+3) (LSB).
// Every table is folded; outputs are Fp3 when the challenge is.
template <int POL, int SEM, u32 M, bool ECH>
__device__ __forceinline__ void fused_body(const RoundArgs& a, u32 bid, u32 nb) {
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 FULL = (1u << NT) - 1;
    constexpr u32 MO = ECH ? FULL : M;
    using P = Policy<POL, MO>;
    P acc;
    acc.init();
    F3 rr;
    Mul3 r = load_challenge_mul(a, rr);
    if (!ECH) r = mul3_prepare<false>(rr);
    const u64 Q = a.L >> 2;
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    F3 lo[3], hi[3];
    // LSB: 16-byte loads and stores when every component array is aligned
    bool vec = false;
    if (SEM == SEM_LSB) {
        uintptr_t bits = 0;
#pragma unroll
        for (int t = 0; t < NT; t++)
            for (int c = 0; c < 3; c++) bits |= (uintptr_t)a.t[t].in[c] | (uintptr_t)a.t[t].out[c];
        vec = (bits & 15) == 0;
    }
    for (u64 k = tid; k < Q; k += stride) {
#pragma unroll
        for (int t = 0; t < NT; t++) {
            const bool EI = ext_of<M>(t);
            F3 x0, x1, x2, x3;
            if (SEM == SEM_LSB) {
                if (vec) {
                    // entries 4k .. 4k+3 of each component as two 16-byte loads
                    ulonglong2 v[3][2];
#pragma unroll
                    for (int c = 0; c < (EI ? 3 : 1); c++) {
                        v[c][0] = ((const ulonglong2*)a.t[t].in[c])[2 * k];
                        v[c][1] = ((const ulonglong2*)a.t[t].in[c])[2 * k + 1];
                    }
                    x0 = f3_make(v[0][0].x, EI ? v[1][0].x : 0, EI ? v[2][0].x : 0);
                    x1 = f3_make(v[0][0].y, EI ? v[1][0].y : 0, EI ? v[2][0].y : 0);
                    x2 = f3_make(v[0][1].x, EI ? v[1][1].x : 0, EI ? v[2][1].x : 0);
                    x3 = f3_make(v[0][1].y, EI ? v[1][1].y : 0, EI ? v[2][1].y : 0);
                }
                else if (EI) { x0 = ld<true>(a.t[t].in, 4 * k); x1 = ld<true>(a.t[t].in, 4 * k + 1); x2 = ld<true>(a.t[t].in, 4 * k + 2); x3 = ld<true>(a.t[t].in, 4 * k + 3); }
                else { x0 = ld<false>(a.t[t].in, 4 * k); x1 = ld<false>(a.t[t].in, 4 * k + 1); x2 = ld<false>(a.t[t].in, 4 * k + 2); x3 = ld<false>(a.t[t].in, 4 * k + 3); }
                if (EI) { lo[t] = f3_fold<true, true>(x0, x1, r); hi[t] = f3_fold<true, true>(x2, x3, r); }
                else if (ECH) { lo[t] = f3_fold<false, true>(x0, x1, r); hi[t] = f3_fold<false, true>(x2, x3, r); }
                else { lo[t] = f3_fold<false, false>(x0, x1, r); hi[t] = f3_fold<false, false>(x2, x3, r); }
                if (vec) {
                    ((ulonglong2*)a.t[t].out[0])[k] = make_ulonglong2(lo[t].c0, hi[t].c0);
                    if (ext_of<MO>(t)) {
                        ((ulonglong2*)a.t[t].out[1])[k] = make_ulonglong2(lo[t].c1, hi[t].c1);
                        ((ulonglong2*)a.t[t].out[2])[k] = make_ulonglong2(lo[t].c2, hi[t].c2);
                    }
                }
                else if (ext_of<MO>(t)) { st<true>(a.t[t].out, 2 * k, lo[t]); st<true>(a.t[t].out, 2 * k + 1, hi[t]); }
                else { st<false>(a.t[t].out, 2 * k, lo[t]); st<false>(a.t[t].out, 2 * k + 1, hi[t]); }
            } else {
                if (EI) { x0 = ld<true>(a.t[t].in, k); x1 = ld<true>(a.t[t].in, k + Q); x2 = ld<true>(a.t[t].in, k + 2 * Q); x3 = ld<true>(a.t[t].in, k + 3 * Q); }
                else { x0 = ld<false>(a.t[t].in, k); x1 = ld<false>(a.t[t].in, k + Q); x2 = ld<false>(a.t[t].in, k + 2 * Q); x3 = ld<false>(a.t[t].in, k + 3 * Q); }
                if (EI) { lo[t] = f3_fold<true, true>(x0, x2, r); hi[t] = f3_fold<true, true>(x1, x3, r); }
                else if (ECH) { lo[t] = f3_fold<false, true>(x0, x2, r); hi[t] = f3_fold<false, true>(x1, x3, r); }
                else { lo[t] = f3_fold<false, false>(x0, x2, r); hi[t] = f3_fold<false, false>(x1, x3, r); }
                if (ext_of<MO>(t)) { st<true>(a.t[t].out, k, lo[t]); st<true>(a.t[t].out, k + Q, hi[t]); }
                else { st<false>(a.t[t].out, k, lo[t]); st<false>(a.t[t].out, k + Q, hi[t]); }
            }
        }
        acc.pair(lo, hi);
    }
    F3 raw[P::NRAW];
    acc.result(raw);
    reduce_and_finalize_seg<P::NRAW>(raw, a, POL, nb, bid);
}
template <int POL, int SEM, u32 M, bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_fused(RoundArgs a) {
    chain_enter();
    fused_body<POL, SEM, M, ECH>(a, blockIdx.x, gridDim.x);
}
// The degree-3 product evaluator.  POL_C3 (four points, the per-round
// path's h(1) included) does not fit 128 registers: one block per SM.
// POL_C3W (the device protocol's three points, each an Fp3 x Fp3 sum in
// three accumulators with the multiplier prepared by W) fits at two blocks
// per SM without spills in MSB order (measured at one block: 8 warps per
// SM, issue 38 %, ALU pipe 45 %).
constexpr int wide_min_blocks(int pol) { return pol == POL_C3W ? 2 : 1; }
template <int POL, int SEM, u32 M, bool ECH>
__global__ void __launch_bounds__(TPB, wide_min_blocks(POL)) k_fused_wide(RoundArgs a) {
    chain_enter();
    fused_body<POL, SEM, M, ECH>(a, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// TMA-staged fused round (MSB or LSB, L a power of two, Q = L/4 a multiple
// of TQ).  Each block owns tiles tile = blockIdx.x + i * gridDim.x of TQ
// quadruples.  Thread 0 streams a tile's 4 quarters (MSB) or its 4 TQ
// consecutive entries (LSB) x components x tables into one shared
// memory stage with cp.async.bulk (one bulk copy per contiguous chunk), the
// stage's mbarrier counting the bytes; TMA_S stages are kept in flight while
// every thread folds and evaluates the quadruple it owns from shared memory
// and stores the folded pair straight to global memory.  Waits are bounded
// by the global timer: after 1 s the block records a timeout in a.status,
// waits (bounded) for its copies in flight and stops.
// ---------------------------------------------------------------------------
constexpr int TQ = TPB;

__device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(u64* bar, u32 count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(u64* bar, u32 bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, u32 bytes, u64* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(u64* bar, u32 phase) {
    u32 ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
    return ok != 0;
}
__device__ __forceinline__ u64 global_ns() {
    u64 t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Wait for phase `phase` of `bar`; false after `limit_ns` (default 1 s).
__device__ __forceinline__ bool mbar_wait_bounded(u64* bar, u32 phase, u64 limit_ns = 1000000000ULL) {
    if (mbar_try_wait(bar, phase)) return true;
    const u64 t0 = global_ns();
    while (!mbar_try_wait(bar, phase))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

template <u32 M, int NT>
struct TmaLayout {
    __host__ __device__ static constexpr int nc(int t) { return ((M >> t) & 1u) ? 3 : 1; }
    // word offset of (table t, quarter q, component c) inside a stage
    __host__ __device__ static constexpr int off(int t, int q, int c) {
        int o = 0;
        for (int u = 0; u < t; u++) o += 4 * nc(u);
        return (o + q * nc(t) + c) * TQ;
    }
    // LSB: the tile's 4 TQ consecutive entries of (table t, component c)
    __host__ __device__ static constexpr int offl(int t, int c) {
        int o = 0;
        for (int u = 0; u < t; u++) o += 4 * nc(u);
        return (o + 4 * c) * TQ;
    }
    __host__ __device__ static constexpr int words() {
        int o = 0;
        for (int u = 0; u < NT; u++) o += 4 * nc(u);
        return o * TQ;
    }
    __host__ __device__ static constexpr int stages() { return words() * 8 <= 24 * 1024 ? 4 : 2; }
    __host__ __device__ static constexpr int smem_bytes() { return words() * 8 * stages(); }
};

template <int POL, int SEM, u32 M, bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_fused_tma(RoundArgs a, u32 ntiles) {
    chain_enter();
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 FULL = (1u << NT) - 1;
    constexpr u32 MO = ECH ? FULL : M;
    using P = Policy<POL, MO>;
    using LAY = TmaLayout<M, NT>;
    constexpr int S = LAY::stages();
    constexpr int SW = LAY::words();
    extern __shared__ __align__(128) u64 tma_smem[];
    __shared__ __align__(8) u64 full_bar[4];
    __shared__ u32 reads_done[4];     // warps done reading the stage's current tile
    __shared__ u32 issued_cnt[4];     // tiles issued into each stage

    const u64 Q = a.L >> 2;
    const u32 G = gridDim.x;
    const int lane = threadIdx.x & 31;
    auto issue = [&](u32 tile, int s) {
        mbar_expect_tx(&full_bar[s], (u32)(SW * 8));
        u64* dst = tma_smem + (size_t)s * SW;
        if (SEM == SEM_LSB) {
            // entries 4 TQ tile .. 4 TQ (tile + 1) - 1, one copy per component
#pragma unroll
            for (int t = 0; t < NT; t++)
#pragma unroll
                for (int c = 0; c < LAY::nc(t); c++)
                    tma_load_1d(dst + LAY::offl(t, c), a.t[t].in[c] + (u64)tile * 4 * TQ, 4 * TQ * 8, &full_bar[s]);
        } else {
#pragma unroll
            for (int t = 0; t < NT; t++)
#pragma unroll
                for (int q = 0; q < 4; q++)
#pragma unroll
                    for (int c = 0; c < LAY::nc(t); c++)
                        tma_load_1d(dst + LAY::off(t, q, c), a.t[t].in[c] + q * Q + (u64)tile * TQ, TQ * 8, &full_bar[s]);
        }
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full_bar[s], 1);
            reads_done[s] = 0;
            issued_cnt[s] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the tile of iteration j goes to stage j % S; keep S tiles in flight
        for (int s = 0; s < S; s++) {
            u32 tile = blockIdx.x + s * G;
            if (tile < ntiles) { issue(tile, s); issued_cnt[s]++; }
        }
    }
    __syncthreads();
    P acc;
    acc.init();
    F3 rr;
    Mul3 r = load_challenge_mul(a, rr);
    if (!ECH) r = mul3_prepare<false>(rr);
    F3 lo[3], hi[3];
    bool abort = false;
    u32 i = 0;
    for (u32 tile = blockIdx.x; tile < ntiles; tile += G, i++) {
        const int s = i % S;
        if (!mbar_wait_bounded(&full_bar[s], (i / S) & 1u)) { abort = true; break; }
        const u64* st_ = tma_smem + (size_t)s * SW;
        const u64 k = (u64)tile * TQ + threadIdx.x;
#pragma unroll
        for (int t = 0; t < NT; t++) {
            F3 x[4];
            if (SEM == SEM_LSB) {
                // entries 4i .. 4i+3 of the tile, two 16-byte loads per component
                u64 w[3][4];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if (c < LAY::nc(t)) {
                        const ulonglong2* p = (const ulonglong2*)(st_ + LAY::offl(t, c)) + 2 * threadIdx.x;
                        const ulonglong2 v0 = p[0], v1 = p[1];
                        w[c][0] = v0.x; w[c][1] = v0.y; w[c][2] = v1.x; w[c][3] = v1.y;
                    } else {
                        w[c][0] = w[c][1] = w[c][2] = w[c][3] = 0;
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; q++) x[q] = f3_make(w[0][q], w[1][q], w[2][q]);
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    x[q].c0 = st_[LAY::off(t, q, 0) + threadIdx.x];
                    if (LAY::nc(t) == 3) {
                        x[q].c1 = st_[LAY::off(t, q, 1) + threadIdx.x];
                        x[q].c2 = st_[LAY::off(t, q, 2) + threadIdx.x];
                    } else {
                        x[q].c1 = x[q].c2 = 0;
                    }
                }
            }
            if (t == NT - 1) {
                // this warp is done with the stage; the last warp to finish
                // reading refills it with the tile of iteration i + S
                __syncwarp();
                if (lane == 0) {
                    __threadfence_block();
                    if (atomicAdd(&reads_done[s], 1u) == NWARP - 1) {
                        atomicExch(&reads_done[s], 0u);
                        const u32 nt = blockIdx.x + (i + S) * G;
                        if (nt < ntiles) {
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            issue(nt, s);
                            issued_cnt[s]++;
                        }
                    }
                }
            }
            // MSB pairs (k, k + 2Q) and (k + Q, k + 3Q); LSB pairs (4i, 4i+1) and (4i+2, 4i+3)
            constexpr int PB = SEM == SEM_LSB ? 1 : 2, HA = SEM == SEM_LSB ? 2 : 1;
            if (ext_of<M>(t)) { lo[t] = f3_fold<true, true>(x[0], x[PB], r); hi[t] = f3_fold<true, true>(x[HA], x[HA + PB], r); }
            else if (ECH) { lo[t] = f3_fold<false, true>(x[0], x[PB], r); hi[t] = f3_fold<false, true>(x[HA], x[HA + PB], r); }
            else { lo[t] = f3_fold<false, false>(x[0], x[PB], r); hi[t] = f3_fold<false, false>(x[HA], x[HA + PB], r); }
            if (SEM == SEM_LSB) {
                // folded entries 2k, 2k+1: one 16-byte store per component
                ((ulonglong2*)a.t[t].out[0])[k] = make_ulonglong2(lo[t].c0, hi[t].c0);
                if (ext_of<MO>(t)) {
                    ((ulonglong2*)a.t[t].out[1])[k] = make_ulonglong2(lo[t].c1, hi[t].c1);
                    ((ulonglong2*)a.t[t].out[2])[k] = make_ulonglong2(lo[t].c2, hi[t].c2);
                }
            } else if (ext_of<MO>(t)) { st<true>(a.t[t].out, k, lo[t]); st<true>(a.t[t].out, k + Q, hi[t]); }
            else { st<false>(a.t[t].out, k, lo[t]); st<false>(a.t[t].out, k + Q, hi[t]); }
        }
        acc.pair(lo, hi);
    }
    if (__syncthreads_or(abort)) {
        // drain the copies in flight (bounded): stage s has completed
        // consumed(s) phases and holds issued_cnt[s] - consumed(s) more
        if (threadIdx.x == 0) {
            for (int s = 0; s < S; s++)
                for (u32 ph = i / S + (s < (int)(i % S) ? 1u : 0u); ph < issued_cnt[s]; ph++)
                    mbar_wait_bounded(&full_bar[s], ph & 1u);
            if (a.status) *(volatile u32*)a.status = EFFSC_STATUS_TIMEOUT;
        }
        return;
    }
    F3 raw[P::NRAW];
    acc.result(raw);
    reduce_and_finalize<P::NRAW>(raw, a, POL);
}

// Fold one table (t) with no evaluation: the unfused path, the last fold of
// finalize(), and the standalone fold.
template <int SEM, bool EI, bool ECH>
__global__ void __launch_bounds__(TPB) k_fold(RoundArgs a, int t) {
    chain_enter();
    constexpr bool EO = EI || ECH;
    F3 rr;
    Mul3 r = load_challenge_mul(a, rr);
    if (!ECH) r = mul3_prepare<false>(rr);
    const u64 L = a.L;
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    const u64* const* in = a.t[t].in;
    u64* const* out = a.t[t].out;
    if (SEM == SEM_MSB_PAD) {
        const u64 half = next_pow2_dev(L) >> 1, paired = L - half;
        // (1 - w) prepared for the tail
        F3 om = f3_sub<ECH>(f3_make(1, 0, 0), rr);
        Mul3 omm = mul3_prepare<ECH>(om);
        for (u64 j = tid; j < half; j += stride) {
            F3 x0 = ld<EI>(in, j);
            F3 y;
            if (j < paired) y = f3_fold<EI, ECH>(x0, ld<EI>(in, j + half), r);
            else y = f3_mul_add<EI, ECH, false, false>(x0, omm, f3_zero());
            st<EO>(out, j, y);
        }
    } else if (SEM == SEM_MSB_FLOOR) {
        const u64 half = L / 2;
        for (u64 j = tid; j < half; j += stride)
            st<EO>(out, j, f3_fold<EI, ECH>(ld<EI>(in, j), ld<EI>(in, j + half), r));
    } else {
        const u64 half = L / 2;
        for (u64 j = tid; j < half; j += stride)
            st<EO>(out, j, f3_fold<EI, ECH>(ld<EI>(in, 2 * j), ld<EI>(in, 2 * j + 1), r));
    }
}

// EqFactored left phase (src/provers/eq_factored.rs:139-172):
//   q0   = sum_a eq_l_lo[a] * sum_b eq_r[b] p_lo[a m + b]
//   qinf = sum_a (eq_l_hi[a] - eq_l_lo[a]) * sum_b eq_r[b] (p_hi - p_lo)[a m + b]
// Tables: t[0] = p, t[1] = eq_l (already folded), t[2] = eq_r.
// M bit 0: p is Fp3, bit 1: eq tables are Fp3.  FUSED: fold p first (MSB,
// L a power of two >= 4) and evaluate on the folded table.
// When an a-block (m = |eq_r| entries of p) spans at least a block's worth of
// threads, a block walks chunks of C = min(m, 4096) consecutive entries: the
// inner sums over b are accumulated unreduced per thread and multiplied by
// eq_l once per chunk, as the split-value structure intends (2 products per
// entry instead of 4).  Smaller m multiplies per entry.
template <bool FUSED, u32 M, bool ECH>
__global__ void __launch_bounds__(TPB) k_eqf_left(RoundArgs a) {
    constexpr bool EPI = ext_of<M>(0), EE = ext_of<M>(1);
    constexpr bool EP = FUSED ? (EPI || ECH) : EPI;     // p after the fold
    constexpr bool ET = EE || EP;
    ProdAcc<EE, ET> q0, qi;
    q0.init();
    qi.init();
    F3 rr;
    Mul3 r = load_challenge_mul(a, rr);
    if (!ECH) r = mul3_prepare<false>(rr);
    const u64 L = a.L;
    const u64 ph = FUSED ? (L >> 2) : (L >> 1);           // half of the (folded) p
    const u64 eh = a.el_len >> 1;
    const u64 mmask = (1ULL << a.m_shift) - 1;
    const u64 m = mmask + 1;
    if (m >= TPB && ph >= m) {
        const u64 C = m < 4096 ? m : 4096;
        const u64 nchunks = ph / C;
        F3 s0t = f3_zero(), sdt = f3_zero();
        for (u64 c = blockIdx.x; c < nchunks; c += gridDim.x) {
            ProdAcc<EE, EP> s0, sd;
            s0.init();
            sd.init();
            const u64 base = c * C;
            // U entries per thread per step, all loads issued before the
            // arithmetic (each entry is read and written by this thread only)
            constexpr int U = (FUSED && EPI) ? 2 : 4;
            constexpr int NX = FUSED ? 4 : 2;
            for (u64 k0 = base + threadIdx.x; k0 < base + C; k0 += (u64)U * TPB) {
                F3 X[U][NX];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const u64 k = k0 + (u64)u * TPB;
                    if (k < base + C)
#pragma unroll
                        for (int j = 0; j < NX; j++) X[u][j] = ld<EPI>(a.t[0].in, k + j * ph);
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const u64 k = k0 + (u64)u * TPB;
                    if (k >= base + C) break;
                    F3 pl, phv;
                    if (FUSED) {
                        if (EPI) { pl = f3_fold<true, true>(X[u][0], X[u][2], r); phv = f3_fold<true, true>(X[u][1], X[u][3], r); }
                        else if (ECH) { pl = f3_fold<false, true>(X[u][0], X[u][2], r); phv = f3_fold<false, true>(X[u][1], X[u][3], r); }
                        else { pl = f3_fold<false, false>(X[u][0], X[u][2], r); phv = f3_fold<false, false>(X[u][1], X[u][3], r); }
                        st<EP>(a.t[0].out, k, pl);
                        st<EP>(a.t[0].out, k + ph, phv);
                    } else {
                        pl = X[u][0];
                        phv = X[u][1];
                    }
                    const F3 er = ld<EE>(a.t[2].in, k & mmask);
                    s0.mac(er, pl);
                    sd.mac(er, f3_sub<EP>(phv, pl));
                }
            }
            const u64 ai = base >> a.m_shift;
            const F3 el = ld<EE>(a.t[1].in, ai), eh_ = ld<EE>(a.t[1].in, ai + eh);
            s0t = f3_add<true>(s0t, f3_mul<EE, ET>(el, s0.result()));
            sdt = f3_add<true>(sdt, f3_mul<EE, ET>(f3_sub<EE>(eh_, el), sd.result()));
        }
        F3 raw[2] = {s0t, sdt};
        reduce_and_finalize<2>(raw, a, POL_EQFL);
        return;
    }
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)gridDim.x * TPB;
    for (u64 k = tid; k < ph; k += stride) {
        F3 pl, phv;
        if (FUSED) {
            F3 x0 = ld<EPI>(a.t[0].in, k), x1 = ld<EPI>(a.t[0].in, k + ph);
            F3 x2 = ld<EPI>(a.t[0].in, k + 2 * ph), x3 = ld<EPI>(a.t[0].in, k + 3 * ph);
            if (EPI) { pl = f3_fold<true, true>(x0, x2, r); phv = f3_fold<true, true>(x1, x3, r); }
            else if (ECH) { pl = f3_fold<false, true>(x0, x2, r); phv = f3_fold<false, true>(x1, x3, r); }
            else { pl = f3_fold<false, false>(x0, x2, r); phv = f3_fold<false, false>(x1, x3, r); }
            st<EP>(a.t[0].out, k, pl);
            st<EP>(a.t[0].out, k + ph, phv);
        } else {
            pl = ld<EPI>(a.t[0].in, k);
            phv = ld<EPI>(a.t[0].in, k + ph);
        }
        const u64 ai = k >> a.m_shift, bi = k & mmask;
        F3 er = ld<EE>(a.t[2].in, bi);
        F3 t0 = f3_mul<EE, EP>(er, pl);
        F3 td = f3_mul<EE, EP>(er, f3_sub<EP>(phv, pl));
        F3 el = ld<EE>(a.t[1].in, ai), eh_ = ld<EE>(a.t[1].in, ai + eh);
        q0.mac(el, t0);
        qi.mac(f3_sub<EE>(eh_, el), td);
    }
    F3 raw[2];
    raw[0] = q0.result();
    raw[1] = qi.result();
    reduce_and_finalize<2>(raw, a, POL_EQFL);
}

}  // namespace effsc
