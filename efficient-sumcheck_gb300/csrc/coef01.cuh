// coef01.cuh -- rounds 0-2 of a Coefficient proof with the degree-3 product
// evaluator (three tables: table 0 in Fp or Fp3, tables 1 and 2 in Fp; Fp3
// challenges) in two passes over the input tables.
//
// Write a quadruple of a table as t_uv, u the variable bound in round 0 and v
// the one bound in round 1 (MSB: entry k + u L/2 + v L/4; LSB: entry
// 4k + u + 2v), and F(y, x) = t00 + y d10 + x d01 + x y d11 (d10 = t10 - t00,
// d01 = t01 - t00, d11 = t11 - t10 - t01 + t00) its bilinear form: after the
// fold with r0 the round-1 pair of the quadruple is (F(r0, 0), F(r0, 1)) and
// after the folds with r0 and r1 its entry is F(r0, r1)
// (src/provers/coefficient.rs:131-140 applied twice; coefficient_lsb.rs for
// the LSB pairs).  The round polynomials are sums of products of three such
// forms (src/tests adversarial evaluator eq * f * g,
// tests/adversarial_verifier.rs:444-466):
//   round 0: h0(u) = sum_k P(u, 0) + P(u, 1), P(y, x) = prod_T F_T(y, x);
//   round 1: h1(x) = sum_k P(r0, x), for each x a cubic in r0.
// The wire of a cubic round is [h(0), h(inf), h(2)] (src/provers/coefficient.rs
// :272-294), so one pass accumulates P at 15 points -- (y, x) in
// {0, 1, 2, inf} x {0, 2, inf} (inf: the leading coefficient) and (u, 1) for
// u in {0, 2, inf} -- and its last block interpolates round 1's three cubics
// at r0 (values at 0, 1, 2 and the leading coefficient).  The second pass
// reads the tables again, folds every quadruple with r0 and r1 at once
// (F(r0, r1): three products by r0, r1 and r0 r1), writes the Fp3 tables of
// length L/4 and evaluates round 2 on them.  Against one pass per round this
// skips writing and re-reading the Fp3 tables of length L/2.
#pragma once
#include "round_common.cuh"

namespace effsc {

constexpr int C301_WORDS = 45;   // 15 points x 3 components
constexpr int C301_STRIDE = 48;  // partial words per block
constexpr int C301_NG = 4;       // point groups (a column of four points each)
constexpr int C301_GT = TPB / C301_NG;   // threads per point group

// The bilinear form of one table's quadruple.
struct CForm {
    F3 t00, d10, d01, d11;
};
template <bool E>
__device__ __forceinline__ CForm cform(const F3& t00, const F3& t01, const F3& t10, const F3& t11) {
    CForm f;
    f.t00 = t00;
    f.d10 = f3_sub<E>(t10, t00);
    f.d01 = f3_sub<E>(t01, t00);
    f.d11 = f3_add<E>(f3_sub<E>(f3_sub<E>(t11, t10), t01), t00);
    return f;
}

template <bool E, bool LSB>
__device__ __forceinline__ F3 c301_ld(const TabIO& T, u64 k, u64 Q, int u, int v) {
    return ld<E>(T.in, LSB ? 4 * k + u + 2 * v : k + (2 * u + v) * Q);
}
template <bool E, bool LSB>
__device__ __forceinline__ void c301_load(F3 (&t)[4], const TabIO& T, u64 k, u64 Q) {
#pragma unroll
    for (int uv = 0; uv < 4; uv++) t[uv] = c301_ld<E, LSB>(T, k, Q, uv >> 1, uv & 1);   // t[2u + v] = t_uv
}

// One column of points for one table: F(y, x) for fixed x is a + y b, so the
// values at y = 0, 1, 2 and the leading coefficient (inf) are a, a + b,
// a + 2b and b.  Column c: 0 is x = 0 (a = t00, b = t10 - t00), 1 is x = 2
// (a = t00 + 2 d01, b = d10 + 2 d11), 2 is x = inf (a = d01, b = d11), 3 is
// x = 1 at y = 0, 2, inf (a = t01, b = t11 - t01).  Loads only the entries
// the column reads.
template <bool E, bool LSB, int C>
__device__ __forceinline__ void c301_column(F3 (&v)[4], const TabIO& T, u64 k, u64 Q) {
    F3 a, b;
    if (C == 0) {
        a = c301_ld<E, LSB>(T, k, Q, 0, 0);
        b = f3_sub<E>(c301_ld<E, LSB>(T, k, Q, 1, 0), a);
    } else if (C == 3) {
        a = c301_ld<E, LSB>(T, k, Q, 0, 1);
        b = f3_sub<E>(c301_ld<E, LSB>(T, k, Q, 1, 1), a);
    } else {
        F3 t[4];
        c301_load<E, LSB>(t, T, k, Q);
        const CForm f = cform<E>(t[0], t[1], t[2], t[3]);
        if (C == 1) {
            a = f3_add<E>(f.t00, f3_add<E>(f.d01, f.d01));
            b = f3_add<E>(f.d10, f3_add<E>(f.d11, f.d11));
        } else {
            a = f.d01;
            b = f.d11;
        }
    }
    v[0] = a;
    v[1] = f3_add<E>(a, b);
    v[2] = f3_add<E>(v[1], b);
    v[3] = b;
}
// s[3 j + c] += F0 F1 F2 at the column's points (j = y index; column 3 has
// y = 0, 2, inf in slots 0, 1, 2).
template <bool E0, bool LSB, int C>
__device__ __forceinline__ void c301_group(Acc (&s)[12], const RoundArgs& a, u64 k, u64 Q) {
    F3 v0[4], v1[4], v2[4];
    c301_column<E0, LSB, C>(v0, a.t[0], k, Q);
    c301_column<false, LSB, C>(v1, a.t[1], k, Q);
    c301_column<false, LSB, C>(v2, a.t[2], k, Q);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int y = C == 3 ? (j == 0 ? 0 : j == 1 ? 2 : 3) : j;
        if (C == 3 && j == 3) break;
        const u64 p = gl_mul(v1[y].c0, v2[y].c0);
        acc_mac(s[3 * j], v0[y].c0, p);
        if (E0) {
            acc_mac(s[3 * j + 1], v0[y].c1, p);
            acc_mac(s[3 * j + 2], v0[y].c2, p);
        }
    }
}

static __device__ __noinline__ void finalize_c301(const u64* S, const RoundArgs& a);

// Pass 1.  Four groups of TPB/4 threads take the same quadruples; group c
// accumulates the points of column c (12 accumulators per thread instead of
// 45), loading only the entries that column reads.  Point i = 4 c + j.
template <bool LSB, bool E0>
__device__ __forceinline__ void c301_body(const RoundArgs& a, u32 bid, u32 nb) {
    const int g = threadIdx.x / C301_GT;
    Acc s[12];
#pragma unroll
    for (int i = 0; i < 12; i++) s[i] = acc_zero();
    const u64 Q = a.L >> 2;
    const u64 stride = (u64)nb * C301_GT;
    for (u64 k = (u64)bid * C301_GT + (threadIdx.x % C301_GT); k < Q; k += stride) {
        switch (g) {
        case 0: c301_group<E0, LSB, 0>(s, a, k, Q); break;
        case 1: c301_group<E0, LSB, 1>(s, a, k, Q); break;
        case 2: c301_group<E0, LSB, 2>(s, a, k, Q); break;
        default: c301_group<E0, LSB, 3>(s, a, k, Q); break;
        }
    }
    // block sums: group c's 12 words are points 4c .. 4c+3 (3 components each)
    __shared__ u64 s_red[NWARP][12];
    __shared__ u64 s_fin[5][C301_STRIDE];
    __shared__ u64 s_tot[C301_STRIDE];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 12; j++) {
        u64 v = acc_reduce(s[j]);
#pragma unroll
        for (int off = 16; off; off >>= 1) v = gl_add(v, __shfl_down_sync(0xffffffffu, v, off));
        if (lane == 0) s_red[warp][j] = v;
    }
    __syncthreads();
    constexpr int WPG = C301_GT / 32;   // warps per group
    if (threadIdx.x < C301_WORDS) {
        const int t = threadIdx.x, i = t / 3, c = t % 3, gg = i / 4, j = 3 * (i % 4) + c;
        u64 v = 0;
#pragma unroll
        for (int w = 0; w < WPG; w++) v = gl_add(v, s_red[gg * WPG + w][j]);
        if (nb == 1) s_tot[t] = v;
        else a.partials[(u64)bid * C301_STRIDE + t] = v;
    }
    if (nb > 1) {
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(a.counter, 1u) == nb - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        if (threadIdx.x < 5 * C301_STRIDE) {
            const int part = threadIdx.x / C301_STRIDE, w = threadIdx.x % C301_STRIDE;
            u64 v = 0, v1 = 0;
            if (w < C301_WORDS) {
                u32 b = part;
                for (; b + 5 < nb; b += 10) {
                    v = gl_add(v, __ldcg(&a.partials[(u64)b * C301_STRIDE + w]));
                    v1 = gl_add(v1, __ldcg(&a.partials[(u64)(b + 5) * C301_STRIDE + w]));
                }
                for (; b < nb; b += 5) v = gl_add(v, __ldcg(&a.partials[(u64)b * C301_STRIDE + w]));
            }
            s_fin[part][w] = gl_add(v, v1);
        }
        __syncthreads();
        if (threadIdx.x < C301_WORDS) {
            u64 t = 0;
#pragma unroll
            for (int p = 0; p < 5; p++) t = gl_add(t, s_fin[p][threadIdx.x]);
            s_tot[threadIdx.x] = t;
        }
        if (threadIdx.x == 0) *a.counter = 0;
    }
    __syncthreads();
    if (warp == 0) finalize_c301(s_tot, a);
}

// G(r) of the cubic with G(0) = g0, G(1) = g1, G(2) = g2 and leading
// coefficient ginf: ginf r (r-1)(r-2) + g0 (r-1)(r-2)/2 - g1 r (r-2) +
// g2 r (r-1)/2.  Not inlined (one warp of a cold SM runs it, where code size
// is time).
static __device__ __noinline__ F3 cubic_at(F3 g0, F3 g1, F3 g2, F3 ginf, F3 r) {
    const u64 inv2 = 0x7FFFFFFF80000001ULL;   // (p + 1) / 2
    const F3 r1 = f3_sub<true>(r, f3_make(1, 0, 0)), r2 = f3_sub<true>(r, f3_make(2, 0, 0));
    const F3 A = f3_mul<true, true>(r1, r2), B = f3_mul<true, true>(r, r2), C = f3_mul<true, true>(r, r1);
    F3 t = f3_mul<true, true>(ginf, f3_mul<true, true>(r, A));
    F3 h = f3_add<true>(f3_mul<true, true>(g0, A), f3_mul<true, true>(g2, C));
    h = f3_mul<true, false>(h, f3_make(inv2, 0, 0));
    t = f3_add<true>(t, h);
    return f3_sub<true>(t, f3_mul<true, true>(g1, B));
}

// Rounds 0 and 1 from the 15 sums (S[3 i + c], point i): the wires
// [h(0), h(inf), h(2)], the hook, the challenges (src/runner.rs:39-55).  Run
// by warp 0 of the last block; round 1's three cubics on lanes 0-2.
static __device__ __noinline__ void finalize_c301(const u64* S, const RoundArgs& a) {
    __shared__ u64 s_w[2][9];
    __shared__ u64 s_c[2][3];
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x & 31;
    // round 0: h0(u) = P(u, 0) + P(u, 1); P(u, 0) is point u of column x = 0
    // (points 0, 2, 3 for u = 0, 2, inf), P(u, 1) points 12, 13, 14
    if (lane < 9) {
        const int e = lane / 3, c = lane % 3;          // wire element: h(0), h(inf), h(2)
        const int p0 = e == 0 ? 0 : e == 1 ? 3 : 2, p1 = e == 0 ? 12 : e == 1 ? 14 : 13;
        s_w[0][lane] = gl_add(S[3 * p0 + c], S[3 * p1 + c]);
    }
    __syncwarp();
    DevTranscript* T = (DevTranscript*)a.tx.tx;
    WarpTx w = tx_load(T, lane);
    for (int rd = 0; rd < 2; rd++) {
        if (rd == 1 && lane < 3) {
            // column x = 0, inf, 2 (wire order) is points 4 xi .. 4 xi + 3 with
            // xi = 0, 2, 1: the cubic's values at y = 0, 1, 2 and its leading
            // coefficient, evaluated at r0
            const int xi = lane == 0 ? 0 : lane == 1 ? 2 : 1;
            const u64* G = S + 12 * xi;
            const F3 v = cubic_at(f3_make(G[0], G[1], G[2]), f3_make(G[3], G[4], G[5]), f3_make(G[6], G[7], G[8]),
                                  f3_make(G[9], G[10], G[11]), f3_make(s_c[0][0], s_c[0][1], s_c[0][2]));
            s_w[1][3 * lane] = v.c0; s_w[1][3 * lane + 1] = v.c1; s_w[1][3 * lane + 2] = v.c2;
        }
        __syncwarp();
        tx_send_elems(w, lane, s_w[rd], 3);
        if (a.tx.hook_len) {
            const uint8_t* hk = a.tx.hook;
            tx_absorb(w, lane, a.tx.hook_len, [&](u32 k) -> uint8_t { return hk[k]; });
        }
        tx_challenge(w, lane, s_c[rd], s_scr);
    }
    tx_store(T, w, lane);
    if (lane < 18) a.tx.proof_wire[lane] = s_w[lane / 9][lane % 9];
    if (lane < 6) a.tx.proof_chal[lane] = s_c[lane / 3][lane % 3];
}

// t00 + r0 d10 + r1 d01 + r0 r1 d11 with the three multipliers prepared.
template <bool E>
__device__ __forceinline__ F3 fold2(const CForm& f, const Mul3 (&K)[3]) {
    AccF<FOLD_FORM> c0, c1, c2;
    c0.from(f.t00.c0);
    c1.from(E ? f.t00.c1 : 0);
    c2.from(E ? f.t00.c2 : 0);
    const F3* d[3] = {&f.d10, &f.d01, &f.d11};
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const F3& x = *d[j];
        const Mul3& m = K[j];
        if (E) {
            c0.mac(x.c0, m.m0); c0.mac(x.c1, m.w2); c0.mac(x.c2, m.w1);
            c1.mac(x.c0, m.m1); c1.mac(x.c1, m.m0); c1.mac(x.c2, m.w2);
            c2.mac(x.c0, m.m2); c2.mac(x.c1, m.m1); c2.mac(x.c2, m.m0);
        } else {
            c0.mac(x.c0, m.m0); c1.mac(x.c0, m.m1); c2.mac(x.c0, m.m2);
        }
    }
    return f3_make(c0.reduce(), c1.reduce(), c2.reduce());
}

// Pass 2: item j (MSB: quadruples j and j + Q/2; LSB: 2j and 2j + 1) gives
// the round-2 pair of the Fp3 tables of length Q = L/4 for all three tables;
// round 2 by the device protocol's degree-3 policy.
template <bool LSB, bool E0>
__device__ __forceinline__ void c32x_body(const RoundArgs& a, u32 bid, u32 nb) {
    using P = Policy<POL_C3W, 7>;
    P acc;
    acc.init();
    const F3 r0 = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    const F3 r1 = f3_make(a.chal2_ptr[0], a.chal2_ptr[1], a.chal2_ptr[2]);
    Mul3 K[3];
    K[0] = mul3_prepare<true>(r0);
    K[1] = mul3_prepare<true>(r1);
    K[2] = mul3_prepare<true>(f3_mul<true, true>(r0, r1));
    const u64 Q = a.L >> 2, H = Q >> 1;
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    for (u64 j = tid; j < H; j += stride) {
        F3 lo[3], hi[3];
        const u64 kl = LSB ? 2 * j : j, kh = LSB ? 2 * j + 1 : j + H;
#pragma unroll
        for (int t = 0; t < 3; t++) {
            F3 x[4];
            if (t == 0 && E0) c301_load<true, LSB>(x, a.t[t], kl, Q);
            else c301_load<false, LSB>(x, a.t[t], kl, Q);
            lo[t] = (t == 0 && E0) ? fold2<true>(cform<true>(x[0], x[1], x[2], x[3]), K)
                                   : fold2<false>(cform<false>(x[0], x[1], x[2], x[3]), K);
            if (t == 0 && E0) c301_load<true, LSB>(x, a.t[t], kh, Q);
            else c301_load<false, LSB>(x, a.t[t], kh, Q);
            hi[t] = (t == 0 && E0) ? fold2<true>(cform<true>(x[0], x[1], x[2], x[3]), K)
                                   : fold2<false>(cform<false>(x[0], x[1], x[2], x[3]), K);
            st<true>(a.t[t].out, kl, lo[t]);
            st<true>(a.t[t].out, kh, hi[t]);
        }
        acc.pair(lo, hi);
    }
    F3 raw[P::NRAW];
    acc.result(raw);
    reduce_and_finalize_seg<P::NRAW>(raw, a, POL_C3W, nb, bid);
}

}  // namespace effsc
