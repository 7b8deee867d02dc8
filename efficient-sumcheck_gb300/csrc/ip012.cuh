// ip012.cuh -- InnerProduct rounds 0-3 of an MSB or LSB proof over Fp3
// challenges in two passes over the base tables.
//
// Write an octet of a table as v(t0, t1, t2), t_i the variable bound in round
// i (MSB: entry m + (4 t0 + 2 t1 + t2) L/8; LSB: entry 8m + t0 + 2 t1 + 4 t2),
// and A(u, v; t2) = v(0,0,t2) + u dA + v eA + u v fA the bilinear form whose
// value at (r0, r1) is the entry after the folds with r0 and r1
// (src/inner_product_sumcheck.rs:143-176 applied twice).
//   round 0: q0 = sum v(0,t1,t2) w(0,t1,t2), qinf = sum of the t0 differences
//            (src/provers/inner_product.rs:94-103);
//   round 1: sum_t2 A(r0, 0; t2) B(r0, 0; t2) and sum_t2 A(r0, inf; t2) B(...)
//            are quadratics in r0;
//   round 2: A(r0, r1; 0) B(r0, r1; 0) and the product of the t2 differences
//            are biquadratic in (r0, r1).
// A quadratic is fixed by its values at 0, 1 and its leading coefficient
// ("inf"), a biquadratic by its values on {0, 1, inf}^2, and the value of a
// product of two bilinear forms at such a point is the product of the
// forms' values there (leading coefficients multiply).  So one pass
// accumulates 26 base-field sums, each one product per octet
// (ip012_sums), and the last block interpolates all three rounds' wire
// values at the challenges as it runs the three transcript steps
// (finalize_ip012).  The second pass folds every octet with r0, r1, r2 at
// once -- the multilinear form sum_s D_s prod_{i in s} r_i with D_s the
// octet's finite differences, 7 base x Fp3 products per component --
// writes the Fp3 tables of length L/8 and evaluates round 3 on them.
// Against the two-pass start of rounds 0-2 this skips writing and
// re-reading the length-L/4 Fp3 tables (24 bytes per entry of L).
#pragma once
#include "ip01.cuh"

namespace effsc {

constexpr int IP012_WORDS = 26;   // base-field sums of the first pass
constexpr int IP012_G1 = 14;      // sums of the first warp group (0..13), the rest in the second

// Sums (grid point index g = 3 u + v, u, v in {0, 1, inf}):
//   0..8   P0[g]  = sum A(u,v;0) B(u,v;0)
//   9..11  R1a[u] = sum A(u,0;1) B(u,0;1)
//   12     R0a    = sum A(0,1;1) B(0,1;1)
//   13     R0b    = sum A(inf,1;1) B(inf,1;1)
//   14..22 Pd[g]  = sum dA(u,v) dB(u,v), dA = A(.,.;1) - A(.,.;0)
//   23..25 R1b[u] = sum A(u,inf;1) B(u,inf;1)
// Values of one table's octet are v[4 t0 + 2 t1 + t2].
template <int GROUP>
__device__ __forceinline__ void ip012_sums(Acc* s, const u64 (&x)[8], const u64 (&y)[8]) {
    if (GROUP == 0) {
        // t2 = 0 grid: (0,0) (0,1) (0,inf) (1,0) (1,1) (1,inf) (inf,0) (inf,1) (inf,inf)
        const u64 xa = gl_sub(x[4], x[0]), ya = gl_sub(y[4], y[0]);     // (inf, 0)
        const u64 xb = gl_sub(x[6], x[2]), yb = gl_sub(y[6], y[2]);     // (inf, 1)
        const u64 xc = gl_sub(x[2], x[0]), yc = gl_sub(y[2], y[0]);     // (0, inf)
        const u64 xd = gl_sub(x[6], x[4]), yd = gl_sub(y[6], y[4]);     // (1, inf)
        const u64 xe = gl_sub(xd, xc), ye = gl_sub(yd, yc);             // (inf, inf)
        acc_mac(s[0], x[0], y[0]);
        acc_mac(s[1], x[2], y[2]);
        acc_mac(s[2], xc, yc);
        acc_mac(s[3], x[4], y[4]);
        acc_mac(s[4], x[6], y[6]);
        acc_mac(s[5], xd, yd);
        acc_mac(s[6], xa, ya);
        acc_mac(s[7], xb, yb);
        acc_mac(s[8], xe, ye);
        // t2 = 1 at v = 0 (u = 0, 1, inf), at (0, 1) and at (inf, 1)
        acc_mac(s[9], x[1], y[1]);
        acc_mac(s[10], x[5], y[5]);
        acc_mac(s[11], gl_sub(x[5], x[1]), gl_sub(y[5], y[1]));
        acc_mac(s[12], x[3], y[3]);
        acc_mac(s[13], gl_sub(x[7], x[3]), gl_sub(y[7], y[3]));
    } else {
        // t2 differences on the grid
        const u64 p00 = gl_sub(x[1], x[0]), q00 = gl_sub(y[1], y[0]);
        const u64 p01 = gl_sub(x[3], x[2]), q01 = gl_sub(y[3], y[2]);
        const u64 p10 = gl_sub(x[5], x[4]), q10 = gl_sub(y[5], y[4]);
        const u64 p11 = gl_sub(x[7], x[6]), q11 = gl_sub(y[7], y[6]);
        const u64 p0i = gl_sub(p01, p00), q0i = gl_sub(q01, q00);
        const u64 p1i = gl_sub(p11, p10), q1i = gl_sub(q11, q10);
        acc_mac(s[0], p00, q00);
        acc_mac(s[1], p01, q01);
        acc_mac(s[2], p0i, q0i);
        acc_mac(s[3], p10, q10);
        acc_mac(s[4], p11, q11);
        acc_mac(s[5], p1i, q1i);
        acc_mac(s[6], gl_sub(p10, p00), gl_sub(q10, q00));
        acc_mac(s[7], gl_sub(p11, p01), gl_sub(q11, q01));
        acc_mac(s[8], gl_sub(p1i, p0i), gl_sub(q1i, q0i));
        // t2 = 1 at v = inf (u = 0, 1, inf)
        const u64 e0 = gl_sub(x[3], x[1]), f0 = gl_sub(y[3], y[1]);
        const u64 e1 = gl_sub(x[7], x[5]), f1 = gl_sub(y[7], y[5]);
        acc_mac(s[9], e0, f0);
        acc_mac(s[10], e1, f1);
        acc_mac(s[11], gl_sub(e1, e0), gl_sub(f1, f0));
    }
}

// Octet m of a base table in the v[4 t0 + 2 t1 + t2] order.
template <bool LSB>
__device__ __forceinline__ void load_octet(u64 (&v)[8], const u64* X, u64 m, u64 O) {
    if (LSB) {
        // entries 8m .. 8m+7: v[4 t0 + 2 t1 + t2] = e[t0 + 2 t1 + 4 t2]
        const ulonglong2* X2 = (const ulonglong2*)X + 4 * m;
        const ulonglong2 e01 = X2[0], e23 = X2[1], e45 = X2[2], e67 = X2[3];
        v[0] = e01.x; v[4] = e01.y; v[2] = e23.x; v[6] = e23.y;
        v[1] = e45.x; v[5] = e45.y; v[3] = e67.x; v[7] = e67.y;
    } else {
        // eight slices of the table per octet: read-only loads with a 128-byte
        // L2 fetch hint (the second pass measured 0.404 -> 0.375 ms at n = 26)
#pragma unroll
        for (int j = 0; j < 8; j++) {
            u64 r;
            asm("ld.global.nc.L2::128B.u64 %0, [%1];" : "=l"(r) : "l"(X + m + j * O));
            v[j] = r;
        }
    }
}

// The inverse of load_octet: octet m back to its table positions.
template <bool LSB>
__device__ __forceinline__ void store_octet(const u64 (&v)[8], u64* X, u64 m, u64 O) {
    if (LSB) {
        ulonglong2* X2 = (ulonglong2*)X + 4 * m;
        X2[0] = make_ulonglong2(v[0], v[4]);
        X2[1] = make_ulonglong2(v[2], v[6]);
        X2[2] = make_ulonglong2(v[1], v[5]);
        X2[3] = make_ulonglong2(v[3], v[7]);
    } else {
#pragma unroll
        for (int j = 0; j < 8; j++) X[m + j * O] = v[j];
    }
}

static __device__ __noinline__ void finalize_ip012(const u64* S, const RoundArgs& a);

// Block and grid reduction of the 26 sums (each warp holds its group's
// words), the last block to finish runs finalize_ip012.
__device__ __forceinline__ void ip012_reduce_and_finalize(const Acc (&s)[IP012_G1], int group, const RoundArgs& a,
                                                          u32 nb, u32 bid) {
    __shared__ u64 s_red[NWARP][IP012_G1];
    __shared__ u64 s_fin[NWARP][32];
    __shared__ u64 s_tot[32];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = group == 0 ? IP012_G1 : IP012_WORDS - IP012_G1;
#pragma unroll
    for (int i = 0; i < IP012_G1; i++) {
        if (i < nw) {
            u64 v = acc_reduce(s[i]);
#pragma unroll
            for (int off = 16; off; off >>= 1) v = gl_add(v, __shfl_down_sync(0xffffffffu, v, off));
            if (lane == 0) s_red[warp][i] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < IP012_WORDS) {
        const int g = threadIdx.x < IP012_G1 ? 0 : 1, i = threadIdx.x - g * IP012_G1;
        u64 v = 0;
#pragma unroll
        for (int w = 0; w < NWARP / 2; w++) v = gl_add(v, s_red[g * (NWARP / 2) + w][i]);
        if (nb == 1) s_tot[threadIdx.x] = v;
        else a.partials[(u64)bid * 32 + threadIdx.x] = v;
    }
    if (nb > 1) {
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(a.counter, 1u) == nb - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        // thread t sums word t % 32 over the blocks t / 32, t / 32 + 8, ...
        const int wd = threadIdx.x & 31, part = threadIdx.x >> 5;
        // four independent sums so that four loads are in flight at once
        u64 v = 0;
        if (wd < IP012_WORDS) {
            u64 v1 = 0, v2 = 0, v3 = 0;
            u32 b = part;
            for (; b + 3 * NWARP < nb; b += 4 * NWARP) {
                v = gl_add(v, __ldcg(&a.partials[(u64)b * 32 + wd]));
                v1 = gl_add(v1, __ldcg(&a.partials[(u64)(b + NWARP) * 32 + wd]));
                v2 = gl_add(v2, __ldcg(&a.partials[(u64)(b + 2 * NWARP) * 32 + wd]));
                v3 = gl_add(v3, __ldcg(&a.partials[(u64)(b + 3 * NWARP) * 32 + wd]));
            }
            for (; b < nb; b += NWARP) v = gl_add(v, __ldcg(&a.partials[(u64)b * 32 + wd]));
            v = gl_add(gl_add(v, v1), gl_add(v2, v3));
        }
        s_fin[part][wd] = v;
        __syncthreads();
        if (threadIdx.x < IP012_WORDS) {
            u64 t = 0;
#pragma unroll
            for (int p = 0; p < NWARP; p++) t = gl_add(t, s_fin[p][threadIdx.x]);
            s_tot[threadIdx.x] = t;
        }
        if (threadIdx.x == 0) *a.counter = 0;
    }
    __syncthreads();
    if (a.acc_mode != ACC_NONE) {
        // one chunk of the tables: carry the sums to the next chunk's launch
        if (threadIdx.x < IP012_WORDS) {
            const u64 v = s_tot[threadIdx.x];
            if (a.acc_mode == ACC_FIRST) a.acc[threadIdx.x] = v;
            else if (a.acc_mode == ACC_MID) a.acc[threadIdx.x] = gl_add(a.acc[threadIdx.x], v);
            else s_tot[threadIdx.x] = gl_add(a.acc[threadIdx.x], v);
        }
        if (a.acc_mode != ACC_LAST) return;
        __syncthreads();
    }
    if (warp == 0) finalize_ip012(s_tot, a);
}

// Pass 1.  Warps 0..3 of a block accumulate sums 0..13 and warps 4..7 sums
// 14..25 of the same octets (13-14 accumulators per thread instead of 26);
// the second group's loads of an octet hit what the first group's brought
// into the caches.  The last block interpolates and runs rounds 0-2.
// MIRROR: the tables are in host memory and a.t[0].out[0], a.t[1].out[0]
// are device buffers of the same length; group 0 writes each octet it loads
// there, so the tables cross the host link once and the second pass reads
// HBM.
template <bool LSB, bool MIRROR = false>
__device__ __forceinline__ void ip012_body(const RoundArgs& a, u32 bid, u32 nb) {
    constexpr int HALF = TPB / 2;
    const int group = threadIdx.x >= HALF;
    Acc s[IP012_G1];
#pragma unroll
    for (int i = 0; i < IP012_G1; i++) s[i] = acc_zero();
    const u64 O = a.L >> 3;
    const u64* A = a.t[0].in[0];
    const u64* B = a.t[1].in[0];
    const u64 stride = (u64)nb * HALF;
    for (u64 m = (u64)bid * HALF + (threadIdx.x & (HALF - 1)); m < O; m += stride) {
        u64 x[8], y[8];
        load_octet<LSB>(x, A, m, O);
        load_octet<LSB>(y, B, m, O);
        if (MIRROR && group == 0) {
            store_octet<LSB>(x, a.t[0].out[0], m, O);
            store_octet<LSB>(y, a.t[1].out[0], m, O);
        }
        if (group == 0) ip012_sums<0>(s, x, y);
        else ip012_sums<1>(s, x, y);
    }
    ip012_reduce_and_finalize(s, group, a, nb, bid);
}

// q(r) of the quadratic with q(0) = s0, q(1) = s1 and leading coefficient
// sinf: s0 + r (s1 - s0 - sinf) + r^2 sinf.  Not inlined: the finalize runs
// it on one warp of one block, where straight-line code is bound by
// instruction fetch (a cold SM, one warp): every call site shares this body.
static __device__ __noinline__ F3 quad_at(F3 s0, F3 s1, F3 sinf, F3 r) {
    const F3 c1 = f3_sub<true>(f3_sub<true>(s1, s0), sinf);
    return f3_add<true>(f3_mul<true, true>(f3_add<true>(f3_mul<true, true>(sinf, r), c1), r), s0);
}

// Rounds 0, 1, 2 from the 26 sums: for each, the wire [q0, qinf], the hook,
// the challenge (src/runner.rs:39-55).  Run by warp 0 of the last block.
// The interpolations run on separate lanes as soon as their challenges are
// known, each lane gathering its own quadratic's three values so that all
// of them make one call: after r0, lanes 0-1 evaluate round 1's two
// quadratics and lanes 2-7 the six quadratics in r0 that round 2's
// biquadratics reduce to; after r1, lanes 0-1 finish round 2 with one
// quadratic in r1 each.
static __device__ __noinline__ void finalize_ip012(const u64* S, const RoundArgs& a) {
    __shared__ u64 s_w[3][6];
    __shared__ u64 s_c[3][3];
    __shared__ u64 s_g[2][3][3];   // round 2: [P0 / Pd][v][component], the quadratics in r0 at r0
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        s_w[0][0] = gl_add(gl_add(S[0], S[1]), gl_add(S[9], S[12]));
        s_w[0][1] = 0; s_w[0][2] = 0;
        s_w[0][3] = gl_add(gl_add(S[6], S[7]), gl_add(S[11], S[13]));
        s_w[0][4] = 0; s_w[0][5] = 0;
    }
    __syncwarp();
    DevTranscript* T = (DevTranscript*)a.tx.tx;
    WarpTx w = tx_load(T, lane);
    for (int rd = 0; rd < 3; rd++) {
        if (rd > 0 && lane < (rd == 1 ? 8 : 2)) {
            // this lane's quadratic: values at 0, 1 and its leading coefficient
            F3 q0, q1, qi, r;
            if (rd == 1) {
                r = f3_make(s_c[0][0], s_c[0][1], s_c[0][2]);
                u64 b0, b1, bi;
                if (lane < 2) {
                    // round 1: sum_t2 A(r0, 0; t2) B(.., ..) and A(r0, inf; t2) B(..)
                    const int o = lane == 0 ? 0 : 2, p = lane == 0 ? 9 : 23;
                    b0 = gl_add(S[o], S[p]);
                    b1 = gl_add(S[o + 3], S[p + 1]);
                    bi = gl_add(S[o + 6], S[p + 2]);
                } else {
                    // round 2: the biquadratic's row v (P0 or Pd) as a quadratic in r0
                    const int j = lane - 2, h = j / 3, v = j % 3;
                    const u64* G = S + 14 * h;
                    b0 = G[v]; b1 = G[3 + v]; bi = G[6 + v];
                }
                q0 = f3_make(b0, 0, 0); q1 = f3_make(b1, 0, 0); qi = f3_make(bi, 0, 0);
            } else {
                r = f3_make(s_c[1][0], s_c[1][1], s_c[1][2]);
                q0 = f3_make(s_g[lane][0][0], s_g[lane][0][1], s_g[lane][0][2]);
                q1 = f3_make(s_g[lane][1][0], s_g[lane][1][1], s_g[lane][1][2]);
                qi = f3_make(s_g[lane][2][0], s_g[lane][2][1], s_g[lane][2][2]);
            }
            const F3 q = quad_at(q0, q1, qi, r);
            if (rd == 2 || lane < 2) {
                s_w[rd][3 * lane] = q.c0; s_w[rd][3 * lane + 1] = q.c1; s_w[rd][3 * lane + 2] = q.c2;
            } else {
                const int j = lane - 2, h = j / 3, v = j % 3;
                s_g[h][v][0] = q.c0; s_g[h][v][1] = q.c1; s_g[h][v][2] = q.c2;
            }
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
    if (lane < 18) a.tx.proof_wire[lane] = s_w[lane / 6][lane % 6];
    if (lane < 9) a.tx.proof_chal[lane] = s_c[lane / 3][lane % 3];
}

// Pass 2.  The octet's entry after the folds with r0, r1, r2:
//   D_000 + sum_{s != 0} D_s K_s,  K_s = prod_{i in s} r_i,
// D_s the finite differences of the octet (three butterfly levels of base
// subtractions); 7 products per component into three accumulators and
// three reductions.  K[j] belongs to the difference at index j of the
// v[4 t0 + 2 t1 + t2] order (bit 2: r0, bit 1: r1, bit 0: r2).
struct Fold3K {
    F3 k[8];   // k[0] unused
};
__device__ __forceinline__ Fold3K fold3_prepare(const F3& r0, const F3& r1, const F3& r2) {
    Fold3K K;
    K.k[0] = f3_make(1, 0, 0);
    K.k[4] = r0;
    K.k[2] = r1;
    K.k[1] = r2;
    K.k[6] = f3_mul<true, true>(r0, r1);
    K.k[5] = f3_mul<true, true>(r0, r2);
    K.k[3] = f3_mul<true, true>(r1, r2);
    K.k[7] = f3_mul<true, true>(K.k[6], r2);
    return K;
}
__device__ __forceinline__ F3 fold3(u64 (&v)[8], const Fold3K& K) {
#pragma unroll
    for (int j = 4; j < 8; j++) v[j] = gl_sub(v[j], v[j - 4]);
#pragma unroll
    for (int j = 0; j < 8; j++)
        if (j & 2) v[j] = gl_sub(v[j], v[j - 2]);
#pragma unroll
    for (int j = 0; j < 8; j++)
        if (j & 1) v[j] = gl_sub(v[j], v[j - 1]);
    AccF<FOLD_FORM> c0, c1, c2;
    c0.from(v[0]);
    c1.zero();
    c2.zero();
#pragma unroll
    for (int j = 1; j < 8; j++) {
        c0.mac(v[j], K.k[j].c0);
        c1.mac(v[j], K.k[j].c1);
        c2.mac(v[j], K.k[j].c2);
    }
    return f3_make(c0.reduce(), c1.reduce(), c2.reduce());
}

// MSB: lane item m < O/2 (O = L/8) folds octets m and m + O/2 of both tables
// into entries m and m + O/2 of the Fp3 tables of length O -- round 3's pair.
// LSB: lane item k folds octets 2k and 2k+1 (entries 16k .. 16k+15) into the
// pair (2k, 2k+1).
template <bool LSB>
__device__ __forceinline__ void ip3x_body(const RoundArgs& a, u32 bid, u32 nb) {
    using P = Policy<POL_IP, 3>;
    P acc;
    acc.init();
    const Fold3K K = fold3_prepare(f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]),
                                   f3_make(a.chal_ptr[3], a.chal_ptr[4], a.chal_ptr[5]),
                                   f3_make(a.chal_ptr[6], a.chal_ptr[7], a.chal_ptr[8]));
    const u64 O = a.L >> 3, H = O >> 1;
    const u64 tid = (u64)bid * TPB + threadIdx.x, stride = (u64)nb * TPB;
    F3 lo[2], hi[2];
    for (u64 m = tid; m < H; m += stride) {
#pragma unroll
        for (int t = 0; t < 2; t++) {
            u64 x[8], y[8];
            if (LSB) {
                load_octet<true>(x, a.t[t].in[0], 2 * m, O);
                load_octet<true>(y, a.t[t].in[0], 2 * m + 1, O);
            } else {
                load_octet<false>(x, a.t[t].in[0], m, O);
                load_octet<false>(y, a.t[t].in[0], m + H, O);
            }
            lo[t] = fold3(x, K);
            hi[t] = fold3(y, K);
            if (LSB) {
                ((ulonglong2*)a.t[t].out[0])[m] = make_ulonglong2(lo[t].c0, hi[t].c0);
                ((ulonglong2*)a.t[t].out[1])[m] = make_ulonglong2(lo[t].c1, hi[t].c1);
                ((ulonglong2*)a.t[t].out[2])[m] = make_ulonglong2(lo[t].c2, hi[t].c2);
            } else {
                st<true>(a.t[t].out, m, lo[t]);
                st<true>(a.t[t].out, m + H, hi[t]);
            }
        }
        acc.pair(lo, hi);
    }
    F3 raw[2];
    acc.result(raw);
    reduce_and_finalize_seg<2>(raw, a, POL_IP, nb, bid);
}

// ---------------------------------------------------------------------------
// Staged passes: tiles of both tables stream into S shared-memory stages by
// bulk copies (cp.async.bulk, the stage's mbarrier counting the bytes);
// waits are bounded by the global timer (1 s: the block records a timeout,
// drains its copies in flight and stops); the last warp to finish reading a
// stage refills it with the block's tile S iterations ahead.  Bytes in
// flight then no longer depend on registers per thread.
// ---------------------------------------------------------------------------
template <int S>
struct StageRing {
    u64 bar[S];
    u32 reads_done[S];
    u32 issued[S];
};
template <int S, class Issue>
__device__ __forceinline__ void ring_start(StageRing<S>& R, u32 ntiles, Issue issue) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&R.bar[s], 1);
            R.reads_done[s] = 0;
            R.issued[s] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int s = 0; s < S; s++) {
            const u32 tile = blockIdx.x + s * gridDim.x;
            if (tile < ntiles) { issue(tile, s); R.issued[s]++; }
        }
    }
    __syncthreads();
}
// The warp has read the stage of its i-th tile; the last warp refills it.
template <int S, class Issue>
__device__ __forceinline__ void ring_release(StageRing<S>& R, u32 i, u32 ntiles, Issue issue) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
        const int s = i % S;
        __threadfence_block();
        if (atomicAdd(&R.reads_done[s], 1u) == NWARP - 1) {
            atomicExch(&R.reads_done[s], 0u);
            const u32 nt = blockIdx.x + (i + S) * gridDim.x;
            if (nt < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(nt, s);
                R.issued[s]++;
            }
        }
    }
}
// After a timed-out wait at iteration i: wait (bounded) for every copy still
// in flight (stage s has completed the phases of the tiles before i and holds
// issued[s] minus those), then record the timeout.
template <int S>
__device__ __forceinline__ void ring_drain(StageRing<S>& R, u32 i, u32* status) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++)
            for (u32 ph = i / S + (s < (int)(i % S) ? 1u : 0u); ph < R.issued[s]; ph++)
                mbar_wait_bounded(&R.bar[s], ph & 1u);
        if (status) *(volatile u32*)status = EFFSC_STATUS_TIMEOUT;
    }
}

constexpr int IP012_TQ = 256;    // octets per tile of the first pass (two per thread)
constexpr int IP012_S = 3;       // its stages: 3 x 32 KB
constexpr int IP012_STAGE_WORDS = 2 * 8 * IP012_TQ;
constexpr int IP012_SMEM = IP012_S * IP012_STAGE_WORDS * 8;

// Pass 1, staged.  Tile = IP012_TQ octets; a stage holds, per table, the
// tile's 8 entries of each octet (MSB: 8 chunks, one per j, of TQ words; LSB:
// the 8 TQ consecutive entries).  Warps 0..3 accumulate sums 0..13, warps
// 4..7 sums 14..25, both from the same stage; each thread takes TQ / 128
// octets of a tile, so the stage wait and release are paid once per two
// octets.
template <bool LSB>
__device__ __forceinline__ void ip012_staged_body(const RoundArgs& a, u32 ntiles) {
    extern __shared__ __align__(128) u64 stg[];
    __shared__ StageRing<IP012_S> R;
    constexpr int TQ = IP012_TQ, S = IP012_S, SW = IP012_STAGE_WORDS;
    const u64 O = a.L >> 3;
    const u64* X[2] = {a.t[0].in[0], a.t[1].in[0]};
    auto issue = [&](u32 tile, int s) {
        mbar_expect_tx(&R.bar[s], (u32)(SW * 8));
        u64* dst = stg + (size_t)s * SW;
        tile += a.tile0;
#pragma unroll
        for (int t = 0; t < 2; t++) {
            if (LSB) {
                tma_load_1d(dst + t * 8 * TQ, X[t] + (u64)tile * 8 * TQ, 8 * TQ * 8, &R.bar[s]);
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++)
                    tma_load_1d(dst + (t * 8 + j) * TQ, X[t] + j * O + (u64)tile * TQ, TQ * 8, &R.bar[s]);
            }
        }
    };
    ring_start<S>(R, ntiles, issue);
    constexpr int HALF = TPB / 2, PER = TQ / HALF;
    static_assert(TQ % HALF == 0, "a tile holds whole rows of octets for a warp group");
    const int group = threadIdx.x >= HALF;
    Acc sums[IP012_G1];
#pragma unroll
    for (int i = 0; i < IP012_G1; i++) sums[i] = acc_zero();
    bool abort = false;
    u32 i = 0;
    for (u32 tile = blockIdx.x; tile < ntiles; tile += gridDim.x, i++) {
        if (!mbar_wait_bounded(&R.bar[i % S], (i / S) & 1u)) { abort = true; break; }
        const u64* st_ = stg + (size_t)(i % S) * SW;
#pragma unroll
        for (int h = 0; h < PER; h++) {
            const int ml = (threadIdx.x & (HALF - 1)) + h * HALF;
            u64 x[8], y[8];
            if (LSB) {
                const ulonglong2* px = (const ulonglong2*)(st_ + 8 * ml);
                const ulonglong2* py = (const ulonglong2*)(st_ + 8 * TQ + 8 * ml);
                const ulonglong2 a01 = px[0], a23 = px[1], a45 = px[2], a67 = px[3];
                const ulonglong2 b01 = py[0], b23 = py[1], b45 = py[2], b67 = py[3];
                x[0] = a01.x; x[4] = a01.y; x[2] = a23.x; x[6] = a23.y; x[1] = a45.x; x[5] = a45.y; x[3] = a67.x; x[7] = a67.y;
                y[0] = b01.x; y[4] = b01.y; y[2] = b23.x; y[6] = b23.y; y[1] = b45.x; y[5] = b45.y; y[3] = b67.x; y[7] = b67.y;
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    x[j] = st_[j * TQ + ml];
                    y[j] = st_[(8 + j) * TQ + ml];
                }
            }
            // the stage is free once the tile's last octets are in registers
            if (h == PER - 1) ring_release<S>(R, i, ntiles, issue);
            if (group == 0) ip012_sums<0>(sums, x, y);
            else ip012_sums<1>(sums, x, y);
        }
    }
    if (__syncthreads_or(abort)) {
        ring_drain<S>(R, i, a.status);
        return;
    }
    ip012_reduce_and_finalize(sums, group, a, gridDim.x, blockIdx.x);
}

}  // namespace effsc
