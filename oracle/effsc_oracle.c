/*
 * effsc_oracle.c -- CPU oracle (test infrastructure only; see effsc_oracle.h).
 *
 * Each function names the reference file:line it restates.  Paths are
 * relative to the root of compsec-epfl/efficient-sumcheck.
 *
 * OpenMP parallelises the long loops so that the same code doubles as the
 * timed CPU baseline; field addition is exact, so the reduction order does
 * not change any result.
 */
#include "effsc_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define PAR_MIN 8192

/* ========================================================================== */
/* Goldilocks base field, canonical representation.                             */
/* Semantics follow the AVX-512 backend's add/sub/mul                            */
/* (src/simd_fields/goldilocks/avx512.rs:66-94, 179-252): results are the same */
/* field values; the oracle keeps canonical (not Montgomery) residues.          */
/* ========================================================================== */

static inline uint64_t fp_reduce128(u128 x) {
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    uint64_t hh = hi >> 32, hl = hi & OR_EPS;
    /* x = lo + hl*2^64 + hh*2^96 ;  2^64 = eps, 2^96 = -1 (mod p) */
    uint64_t t0 = lo - hh;
    if (lo < hh) t0 -= OR_EPS;
    uint64_t t1 = hl * OR_EPS;
    uint64_t t2 = t0 + t1;
    if (t2 < t1) t2 += OR_EPS;
    return t2 >= OR_P ? t2 - OR_P : t2;
}

uint64_t or_fp_add(uint64_t a, uint64_t b) {
    uint64_t s = a + b;
    if (s < a) s += OR_EPS;          /* carry: 2^64 = eps (mod p) */
    return s >= OR_P ? s - OR_P : s;
}
uint64_t or_fp_sub(uint64_t a, uint64_t b) {
    uint64_t d = a - b;
    if (a < b) d -= OR_EPS;          /* borrow: -2^64 = -eps (mod p) */
    return d;
}
uint64_t or_fp_mul(uint64_t a, uint64_t b) { return fp_reduce128((u128)a * b); }
static uint64_t fp_pow(uint64_t a, uint64_t e) {
    uint64_t r = 1;
    while (e) { if (e & 1) r = or_fp_mul(r, a); a = or_fp_mul(a, a); e >>= 1; }
    return r;
}
uint64_t or_fp_inv(uint64_t a) { return fp_pow(a, OR_P - 2); }
/* Montgomery form of the crate (src/field.rs:314-375): mont(x) = x*2^64 mod p.
 * 2^64 mod p = eps and 2^-64 mod p = p - 2^32. */
uint64_t or_fp_to_mont(uint64_t a) { return or_fp_mul(a % OR_P, OR_EPS); }
uint64_t or_fp_from_mont(uint64_t a) { return or_fp_mul(a % OR_P, OR_P - (1ULL << 32)); }

/* ---- F = Fp3 = Fp[X]/(X^3 - W) (src/tests/fields.rs:73-100) ----------------- */
static const or_f F_ZERO = {{0, 0, 0}};
static const or_f F_ONE = {{1, 0, 0}};

static inline or_f f_add(or_f a, or_f b) {
    or_f r; for (int i = 0; i < 3; i++) r.c[i] = or_fp_add(a.c[i], b.c[i]); return r;
}
static inline or_f f_sub(or_f a, or_f b) {
    or_f r; for (int i = 0; i < 3; i++) r.c[i] = or_fp_sub(a.c[i], b.c[i]); return r;
}
/* Schoolbook product mod X^3 - W.  arkworks' CubicExtField uses a
 * Karatsuba-style formula; the field values are identical. */
static inline or_f f_mul(or_f a, or_f b) {
    if (!(a.c[1] | a.c[2] | b.c[1] | b.c[2])) {       /* both embedded: one base product */
        or_f r = {{or_fp_mul(a.c[0], b.c[0]), 0, 0}}; return r;
    }
    uint64_t a0 = a.c[0], a1 = a.c[1], a2 = a.c[2], b0 = b.c[0], b1 = b.c[1], b2 = b.c[2];
    or_f r;
    r.c[0] = or_fp_add(or_fp_mul(a0, b0), or_fp_mul(OR_W, or_fp_add(or_fp_mul(a1, b2), or_fp_mul(a2, b1))));
    r.c[1] = or_fp_add(or_fp_add(or_fp_mul(a0, b1), or_fp_mul(a1, b0)), or_fp_mul(OR_W, or_fp_mul(a2, b2)));
    r.c[2] = or_fp_add(or_fp_add(or_fp_mul(a0, b2), or_fp_mul(a1, b1)), or_fp_mul(a2, b0));
    return r;
}
static inline int f_eq(or_f a, or_f b) { return a.c[0] == b.c[0] && a.c[1] == b.c[1] && a.c[2] == b.c[2]; }
static inline or_f f_from_u64(uint64_t x) { or_f r = {{x % OR_P, 0, 0}}; return r; }
static inline or_f f_load(const uint64_t* p) { or_f r = {{p[0], p[1], p[2]}}; return r; }
static inline void f_store(uint64_t* p, or_f a) { p[0] = a.c[0]; p[1] = a.c[1]; p[2] = a.c[2]; }

void or_f3_mul(const uint64_t* a, const uint64_t* b, uint64_t* out) {
    f_store(out, f_mul(f_load(a), f_load(b)));
}

static inline void f_zero_init(or_f* x) { x->c[0] = x->c[1] = x->c[2] = 0; }
#pragma omp declare reduction(fadd : or_f : omp_out = f_add(omp_out, omp_in)) \
    initializer(f_zero_init(&omp_priv))

static inline size_t next_pow2(size_t n) {
    size_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

/* ========================================================================== */
/* Seeded uniform generator (SplitMix64, rejection of values >= p).             */
/* Element i of a stream seeded with s is mix(s + (i+1)*gamma), re-mixed while  */
/* it is >= p (probability 2^-32 per draw), so every index is independent.      */
/* ========================================================================== */
#define SM_GAMMA 0x9E3779B97F4A7C15ULL
uint64_t or_splitmix64_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
uint64_t or_table_seed(uint64_t seed, uint64_t table) {
    return or_splitmix64_mix(seed + (table + 1) * 0x632BE59BD9B4E019ULL);
}
uint64_t or_gen_element(uint64_t seed, uint64_t i) {
    uint64_t z = or_splitmix64_mix(seed + (i + 1) * SM_GAMMA);
    while (z >= OR_P) z = or_splitmix64_mix(z + SM_GAMMA);
    return z;
}
void or_gen_table(uint64_t seed, uint64_t n, uint64_t* out) {
    #pragma omp parallel for schedule(static) if (n > PAR_MIN)
    for (uint64_t i = 0; i < n; i++) out[i] = or_gen_element(seed, i);
}

/* ========================================================================== */
/* Keccak-f[1600] (FIPS 202 section 3) and the transcript duplex sponge.        */
/* The crate's default transcript is spongefish 0.7 (src/transcript/            */
/* spongefish.rs:17-44), which is not available here; this duplex is the        */
/* project's own documented Fiat-Shamir transcript.                             */
/* ========================================================================== */
static const uint64_t KRC[24] = {
    0x0000000000000001ULL, 0x0000000000008082ULL, 0x800000000000808AULL, 0x8000000080008000ULL,
    0x000000000000808BULL, 0x0000000080000001ULL, 0x8000000080008081ULL, 0x8000000000008009ULL,
    0x000000000000008AULL, 0x0000000000000088ULL, 0x0000000080008009ULL, 0x000000008000000AULL,
    0x000000008000808BULL, 0x800000000000008BULL, 0x8000000000008089ULL, 0x8000000000008003ULL,
    0x8000000000008002ULL, 0x8000000000000080ULL, 0x000000000000800AULL, 0x800000008000000AULL,
    0x8000000080008081ULL, 0x8000000000008080ULL, 0x0000000080000001ULL, 0x8000000080008008ULL};
/* rotation offset of lane x + 5y */
static const int KROT[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43,
                             25, 39, 41, 45, 15, 21, 8, 18, 2, 61, 56, 14};
static inline uint64_t rotl64(uint64_t x, int r) { return r ? (x << r) | (x >> (64 - r)) : x; }

void or_keccak_f1600(uint64_t* A) {
    for (int round = 0; round < 24; round++) {
        uint64_t C[5], D[5], B[25];
        for (int x = 0; x < 5; x++) C[x] = A[x] ^ A[x + 5] ^ A[x + 10] ^ A[x + 15] ^ A[x + 20];
        for (int x = 0; x < 5; x++) D[x] = C[(x + 4) % 5] ^ rotl64(C[(x + 1) % 5], 1);
        for (int i = 0; i < 25; i++) A[i] ^= D[i % 5];
        /* rho + pi: B[y, 2x+3y] = rot(A[x, y]) */
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++)
                B[y + 5 * ((2 * x + 3 * y) % 5)] = rotl64(A[x + 5 * y], KROT[x + 5 * y]);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++)
                A[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
        A[0] ^= KRC[round];
    }
}

#define T_RATE 136
static inline void st_xor_byte(uint64_t* st, unsigned i, uint8_t b) {
    st[i >> 3] ^= (uint64_t)b << (8 * (i & 7));
}
static inline uint8_t st_get_byte(const uint64_t* st, unsigned i) {
    return (uint8_t)(st[i >> 3] >> (8 * (i & 7)));
}
size_t or_transcript_size(void) { return sizeof(or_transcript); }

void or_transcript_absorb(or_transcript* t, const uint8_t* data, size_t len) {
    if (t->kind != OR_T_KECCAK) return;
    /* Duplex: the next call's input is XORed into the state that produced the
     * last output; the permutation runs once per absorb->squeeze switch. */
    if (t->squeezing) { t->pos = 0; t->squeezing = 0; }
    for (size_t i = 0; i < len; i++) {
        if (t->pos == T_RATE) { or_keccak_f1600(t->st); t->pos = 0; }
        st_xor_byte(t->st, t->pos++, data[i]);
    }
}
void or_transcript_squeeze(or_transcript* t, uint8_t* out, size_t len) {
    if (!t->squeezing) {
        if (t->pos == T_RATE) { or_keccak_f1600(t->st); t->pos = 0; }
        st_xor_byte(t->st, t->pos, 0x06);
        st_xor_byte(t->st, T_RATE - 1, 0x80);
        or_keccak_f1600(t->st);
        t->pos = 0;
        t->squeezing = 1;
    }
    for (size_t i = 0; i < len; i++) {
        if (t->pos == T_RATE) { or_keccak_f1600(t->st); t->pos = 0; }
        out[i] = st_get_byte(t->st, t->pos++);
    }
}
void or_transcript_init_keccak(or_transcript* t, int deg, const uint8_t* label, size_t len) {
    memset(t, 0, sizeof(*t));
    t->kind = OR_T_KECCAK;
    t->deg = deg;
    uint8_t l8[8];
    for (int i = 0; i < 8; i++) l8[i] = (uint8_t)((uint64_t)len >> (8 * i));
    or_transcript_absorb(t, l8, 8);
    or_transcript_absorb(t, label, len);
}
/* Test transcript: sends are no-ops and a challenge is F::from_u64(next_u64())
 * (src/transcript/sanity.rs:25-45), with SplitMix64 as the generator. */
void or_transcript_init_test(or_transcript* t, int deg, uint64_t seed) {
    memset(t, 0, sizeof(*t));
    t->kind = OR_T_TEST;
    t->deg = deg;
    t->sm = seed;
}
void or_transcript_send(or_transcript* t, const uint64_t* v) {
    if (t->kind != OR_T_KECCAK) return;
    uint8_t buf[24];
    int n = t->deg;
    for (int c = 0; c < n; c++)
        for (int i = 0; i < 8; i++) buf[8 * c + i] = (uint8_t)(v[c] >> (8 * i));
    or_transcript_absorb(t, buf, 8 * (size_t)n);
}
void or_transcript_challenge(or_transcript* t, uint64_t* out) {
    if (t->kind == OR_T_TEST) {
        t->sm += SM_GAMMA;
        uint64_t x = or_splitmix64_mix(t->sm);
        out[0] = x % OR_P; out[1] = 0; out[2] = 0;
        return;
    }
    out[1] = out[2] = 0;
    for (int c = 0; c < t->deg; c++) {
        uint8_t b[16];
        or_transcript_squeeze(t, b, 16);
        uint64_t lo = 0, hi = 0;
        for (int i = 0; i < 8; i++) { lo |= (uint64_t)b[i] << (8 * i); hi |= (uint64_t)b[8 + i] << (8 * i); }
        out[c] = fp_reduce128(((u128)hi << 64) | lo);
    }
}

/* ========================================================================== */
/* Shared table kernels.                                                       */
/* ========================================================================== */

/* In-place half-split fold with implicit zero padding:
 * src/inner_product_sumcheck.rs:143-176 and src/multilinear_sumcheck.rs:132-178
 * (the SIMD reduce_msb_in_place, src/simd_sumcheck/reduce.rs:27-75, has the
 * same semantics). */
static void fold_msb_pad(or_f* v, size_t* len, or_f w) {
    size_t n = *len;
    if (n <= 1) return;
    size_t half = next_pow2(n) >> 1, paired = n - half;
    #pragma omp parallel for schedule(static) if (paired > PAR_MIN)
    for (size_t i = 0; i < paired; i++) v[i] = f_add(v[i], f_mul(f_sub(v[i + half], v[i]), w));
    or_f om = f_sub(F_ONE, w);
    for (size_t i = paired; i < half; i++) v[i] = f_mul(v[i], om);
    *len = half;
}
/* Half-split fold with floor(len/2), no padding: msb_fold_vec,
 * src/provers/coefficient.rs:131-140. */
static void fold_msb_floor(or_f* v, size_t* len, or_f c) {
    size_t n = *len;
    if (n <= 1) return;
    size_t half = n / 2;
    #pragma omp parallel for schedule(static) if (half > PAR_MIN)
    for (size_t k = 0; k < half; k++) v[k] = f_add(v[k], f_mul(c, f_sub(v[k + half], v[k])));
    *len = half;
}
/* Pair-split fold, new[i] = v[2i] + w (v[2i+1] - v[2i]), floor(len/2):
 * src/provers/multilinear_lsb.rs:141-166, inner_product_lsb.rs:78-89,
 * src/reductions/pairwise.rs:46-81. */
static void fold_lsb(or_f** pv, size_t* len, or_f w) {
    size_t n = *len;
    if (n <= 1) return;
    size_t half = n / 2;
    or_f* v = *pv;
    if (half > PAR_MIN) {
        or_f* out = (or_f*)malloc(sizeof(or_f) * half);
        #pragma omp parallel for schedule(static)
        for (size_t i = 0; i < half; i++) out[i] = f_add(v[2 * i], f_mul(w, f_sub(v[2 * i + 1], v[2 * i])));
        free(v);
        *pv = out;
    } else {
        for (size_t i = 0; i < half; i++) v[i] = f_add(v[2 * i], f_mul(w, f_sub(v[2 * i + 1], v[2 * i])));
    }
    *len = half;
}

/* ========================================================================== */
/* Prover construction                                                          */
/* ========================================================================== */
static or_f* load_table(const uint64_t* src, size_t n, int ncomp) {
    or_f* t = (or_f*)calloc(n ? n : 1, sizeof(or_f));
    for (size_t i = 0; i < n; i++) {
        t[i].c[0] = src[(size_t)ncomp * i] % OR_P;
        t[i].c[1] = ncomp == 3 ? src[3 * i + 1] % OR_P : 0;
        t[i].c[2] = ncomp == 3 ? src[3 * i + 2] % OR_P : 0;
    }
    return t;
}

or_prover* or_prover_new(int kind, int order, int deg, int ntab,
                         const uint64_t* const* tables, const size_t* lens, int ncomp) {
    or_prover* p = (or_prover*)calloc(1, sizeof(or_prover));
    p->kind = kind; p->order = order; p->deg = deg; p->ntab = ntab;
    for (int i = 0; i < ntab; i++) {
        p->len[i] = lens[i];
        p->t[i] = load_table(tables[i], lens[i], ncomp);
    }
    p->coef_deg = ntab;
    /* InnerProductProver::new asserts equal lengths
     * (src/provers/inner_product.rs:33-36, inner_product_lsb.rs:31-34). */
    if (kind == OR_IP && lens[0] != lens[1]) p->error = 1;
    return p;
}

/* build_eq_table, src/provers/eq_factored.rs:217-239 (MSB layout). */
static or_f* build_eq(const or_f* w, size_t v) {
    size_t size = (size_t)1 << v;
    or_f* t = (or_f*)malloc(sizeof(or_f) * size);
    for (size_t i = 0; i < size; i++) t[i] = F_ZERO;
    t[0] = F_ONE;
    for (size_t j = 0; j < v; j++) {
        size_t stride = (size_t)1 << (v - 1 - j), block = 2 * stride, populated = (size_t)1 << j;
        for (size_t b = 0; b < populated; b++) {
            size_t base = b * block;
            or_f parent = t[base];
            t[base] = f_mul(parent, f_sub(F_ONE, w[j]));
            t[base + stride] = f_mul(parent, w[j]);
        }
    }
    return t;
}
void or_build_eq_table(const uint64_t* w, size_t v, uint64_t* out) {
    or_f* wf = load_table(w, v, 3);
    or_f* t = build_eq(wf, v);
    for (size_t i = 0; i < ((size_t)1 << v); i++) f_store(out + 3 * i, t[i]);
    free(t); free(wf);
}

/* EqFactoredProver::new, src/provers/eq_factored.rs:90-114. */
or_prover* or_eqf_new(int deg, const uint64_t* w, size_t v, const uint64_t* pv, size_t plen, int ncomp) {
    or_prover* p = (or_prover*)calloc(1, sizeof(or_prover));
    p->kind = OR_EQF; p->order = OR_MSB; p->deg = deg; p->ntab = 3;
    size_t n = (size_t)1 << v;
    if (plen > n) p->error = 1;
    or_f* wf = load_table(w, v, 3);
    p->v = v; p->v_l = v / 2;
    p->t[1] = build_eq(wf, p->v_l);
    p->len[1] = (size_t)1 << p->v_l;
    p->t[2] = build_eq(wf + p->v_l, v - p->v_l);
    p->len[2] = (size_t)1 << (v - p->v_l);
    p->t[0] = (or_f*)malloc(sizeof(or_f) * n);
    or_f* tmp = load_table(pv, plen < n ? plen : n, ncomp);
    for (size_t i = 0; i < n; i++) p->t[0][i] = i < plen ? tmp[i] : F_ZERO;
    p->len[0] = n;
    free(tmp); free(wf);
    return p;
}

/* GkrProver::new, src/provers/gkr.rs:61-82: w_b[b n + c] = W(b),
 * w_c[b n + c] = W(c); the gate tables must have n*n entries (assert). */
or_prover* or_gkr_new(int deg, const uint64_t* add, const uint64_t* mult, const uint64_t* w, size_t n, int ncomp) {
    or_prover* p = (or_prover*)calloc(1, sizeof(or_prover));
    p->kind = OR_GKR; p->order = OR_MSB; p->deg = deg; p->ntab = 4;
    size_t nbc = n * n;
    p->t[0] = load_table(add, nbc, ncomp);
    p->t[1] = load_table(mult, nbc, ncomp);
    or_f* wf = load_table(w, n, ncomp);
    p->t[2] = (or_f*)malloc(sizeof(or_f) * (nbc ? nbc : 1));
    p->t[3] = (or_f*)malloc(sizeof(or_f) * (nbc ? nbc : 1));
    for (size_t b = 0; b < n; b++)
        for (size_t c = 0; c < n; c++) {
            p->t[2][b * n + c] = wf[b];
            p->t[3][b * n + c] = wf[c];
        }
    for (int i = 0; i < 4; i++) p->len[i] = nbc;
    free(wf);
    return p;
}
void or_gkr_claimed_w_values(const or_prover* p, uint64_t* out) {
    or_f wb = F_ZERO, wc = F_ZERO;
    if (p->len[2] == 1) { wb = p->t[2][0]; wc = p->t[3][0]; }
    f_store(out, wb);
    f_store(out + 3, wc);
}

void or_prover_free(or_prover* p) {
    if (!p) return;
    for (int i = 0; i < 4; i++) free(p->t[i]);
    free(p);
}
int or_prover_degree(const or_prover* p) {
    switch (p->kind) {
        case OR_ML: return 1;
        case OR_IP: return 2;
        case OR_COEF: return p->coef_deg;
        default: return 2;
    }
}
size_t or_prover_table_len(const or_prover* p, int i) { return p->len[i]; }
void or_prover_read_table(const or_prover* p, int i, uint64_t* out) {
    for (size_t k = 0; k < p->len[i]; k++) f_store(out + 3 * k, p->t[i][k]);
}

/* ========================================================================== */
/* Round polynomials                                                            */
/* ========================================================================== */

/* MultilinearProver round: compute_sumcheck_polynomial,
 * src/multilinear_sumcheck.rs:86-124 (the fused kernel :189-254 yields the
 * same values as fold-then-compute). */
static void ml_msb_compute(const or_f* v, size_t n, or_f* s0o, or_f* s1o) {
    if (n == 0) { *s0o = F_ZERO; *s1o = F_ZERO; return; }
    if (n == 1) { *s0o = v[0]; *s1o = F_ZERO; return; }
    size_t half = next_pow2(n) >> 1, paired = n - half;
    or_f s0 = F_ZERO, s1 = F_ZERO;
    #pragma omp parallel for reduction(fadd : s0, s1) schedule(static) if (paired > PAR_MIN)
    for (size_t i = 0; i < paired; i++) { s0 = f_add(s0, v[i]); s1 = f_add(s1, v[i + half]); }
    for (size_t i = paired; i < half; i++) s0 = f_add(s0, v[i]);  /* tail, hi implicitly zero */
    *s0o = s0; *s1o = s1;
}
/* compute_lsb, src/provers/multilinear_lsb.rs:60-96. */
static void ml_lsb_compute(const or_f* v, size_t n, or_f* s0o, or_f* s1o) {
    if (n == 0) { *s0o = F_ZERO; *s1o = F_ZERO; return; }
    if (n == 1) { *s0o = v[0]; *s1o = F_ZERO; return; }
    or_f s0 = F_ZERO, s1 = F_ZERO;
    size_t pairs = n / 2;
    #pragma omp parallel for reduction(fadd : s0, s1) schedule(static) if (pairs > PAR_MIN)
    for (size_t k = 0; k < pairs; k++) { s0 = f_add(s0, v[2 * k]); s1 = f_add(s1, v[2 * k + 1]); }
    if (n & 1) s0 = f_add(s0, v[n - 1]);
    *s0o = s0; *s1o = s1;
}
/* InnerProductProver round body, src/provers/inner_product.rs:73-112. */
static void ip_msb_compute(const or_f* a, const or_f* b, size_t n, or_f* q0o, or_f* qio) {
    if (n <= 1) { *q0o = n == 1 ? f_mul(a[0], b[0]) : F_ZERO; *qio = F_ZERO; return; }
    size_t half = next_pow2(n) >> 1, paired = n - half;
    or_f q0 = F_ZERO, qi = F_ZERO, tail = F_ZERO;
    #pragma omp parallel for reduction(fadd : q0, qi) schedule(static) if (paired > PAR_MIN)
    for (size_t i = 0; i < paired; i++) {
        q0 = f_add(q0, f_mul(a[i], b[i]));
        qi = f_add(qi, f_mul(f_sub(a[i + half], a[i]), f_sub(b[i + half], b[i])));
    }
    for (size_t i = paired; i < half; i++) tail = f_add(tail, f_mul(a[i], b[i]));
    *q0o = f_add(q0, tail); *qio = f_add(qi, tail);
}
/* compute_lsb and the fused remainder, src/provers/inner_product_lsb.rs:55-144.
 * Returns -1 where the reference indexes past the end (odd length >= 3 in
 * round 0). */
static int ip_lsb_compute(const or_f* a, const or_f* b, size_t n, int round0, or_f* q0o, or_f* qio) {
    if (n == 0) { *q0o = F_ZERO; *qio = F_ZERO; return 0; }
    if (n == 1) { *q0o = f_mul(a[0], b[0]); *qio = F_ZERO; return 0; }
    if (round0 && (n & 1)) return -1;
    or_f q0 = F_ZERO, qi = F_ZERO;
    size_t pairs = n / 2;
    #pragma omp parallel for reduction(fadd : q0, qi) schedule(static) if (pairs > PAR_MIN)
    for (size_t k = 0; k < pairs; k++) {
        or_f ae = a[2 * k], ao = a[2 * k + 1], be = b[2 * k], bo = b[2 * k + 1];
        q0 = f_add(q0, f_mul(ae, be));
        qi = f_add(qi, f_mul(f_sub(ao, ae), f_sub(bo, be)));
    }
    if (n & 1) q0 = f_add(q0, f_mul(a[n - 1], b[n - 1]));
    *q0o = q0; *qio = qi;
    return 0;
}

/* Product-of-pairwise-tables evaluator (degree k = number of tables):
 * coefficients of prod_i (lo_i + x (hi_i - lo_i)); k = 3 is TripleProductEval
 * (tests/adversarial_verifier.rs:444-466), k = 1 is Degree1Eval
 * (src/provers/coefficient.rs:341-351). */
static void product_accumulate(or_f* coeffs, int k, const or_f* lo, const or_f* hi) {
    or_f c[4] = {F_ONE, F_ZERO, F_ZERO, F_ZERO};
    for (int i = 0; i < k; i++) {
        or_f d = f_sub(hi[i], lo[i]);
        or_f n[4] = {F_ZERO, F_ZERO, F_ZERO, F_ZERO};
        for (int j = 0; j <= i; j++) {
            n[j] = f_add(n[j], f_mul(c[j], lo[i]));
            n[j + 1] = f_add(n[j + 1], f_mul(c[j], d));
        }
        memcpy(c, n, sizeof(c));
    }
    for (int j = 0; j <= k; j++) coeffs[j] = f_add(coeffs[j], c[j]);
}
/* msb_parallel_evaluate (src/provers/coefficient.rs:165-222) and
 * parallel_evaluate (src/coefficient_sumcheck.rs:155-190). */
static void coef_evaluate(const or_prover* p, or_f* coeffs) {
    int k = p->ntab;
    size_t n = p->len[0];
    size_t half = n / 2;
    or_f c0 = F_ZERO, c1 = F_ZERO, c2 = F_ZERO, c3 = F_ZERO;
    #pragma omp parallel for reduction(fadd : c0, c1, c2, c3) schedule(static) if (half > PAR_MIN)
    for (size_t j = 0; j < half; j++) {
        or_f lo[3], hi[3];
        for (int i = 0; i < k; i++) {
            size_t il = p->order == OR_MSB ? j : 2 * j;
            size_t ih = p->order == OR_MSB ? j + half : 2 * j + 1;
            lo[i] = p->t[i][il];
            hi[i] = p->t[i][ih];
        }
        or_f acc[4] = {F_ZERO, F_ZERO, F_ZERO, F_ZERO};
        product_accumulate(acc, k, lo, hi);
        c0 = f_add(c0, acc[0]); c1 = f_add(c1, acc[1]); c2 = f_add(c2, acc[2]); c3 = f_add(c3, acc[3]);
    }
    coeffs[0] = c0; coeffs[1] = c1; coeffs[2] = c2; coeffs[3] = c3;
}
/* eval_poly_at (Horner), src/provers/coefficient.rs:249-259. */
static or_f horner(const or_f* c, int d, or_f x) {
    or_f r = c[d];
    for (int i = d - 1; i >= 0; i--) r = f_add(f_mul(r, x), c[i]);
    return r;
}
static void coef_reduce(or_prover* p, or_f c) {
    for (int i = 0; i < p->ntab; i++) {
        if (p->order == OR_MSB) fold_msb_floor(p->t[i], &p->len[i], c);
        else fold_lsb(&p->t[i], &p->len[i], c);
    }
}

/* EqFactoredProver::round_poly_left, src/provers/eq_factored.rs:139-172. */
static void eqf_left(const or_prover* p, or_f* q0o, or_f* qio) {
    size_t eq_l_half = p->len[1] >> 1, p_half = p->len[0] >> 1, m = p->len[2];
    const or_f *el = p->t[1], *er = p->t[2], *pp = p->t[0];
    or_f q0 = F_ZERO, qi = F_ZERO;
    (void)p_half;
    #pragma omp parallel for reduction(fadd : q0, qi) schedule(static) if (eq_l_half * m > PAR_MIN)
    for (size_t a = 0; a < eq_l_half; a++) {
        or_f in0 = F_ZERO, ind = F_ZERO;
        for (size_t b = 0; b < m; b++) {
            or_f e = er[b], pl = pp[a * m + b], ph = pp[p_half + a * m + b];
            in0 = f_add(in0, f_mul(e, pl));
            ind = f_add(ind, f_mul(e, f_sub(ph, pl)));
        }
        q0 = f_add(q0, f_mul(el[a], in0));
        qi = f_add(qi, f_mul(f_sub(el[eq_l_half + a], el[a]), ind));
    }
    *q0o = q0; *qio = qi;
}
/* EqFactoredProver::round_poly_right, src/provers/eq_factored.rs:178-209. */
static void eqf_right(const or_prover* p, or_f* q0o, or_f* qio) {
    size_t n = p->len[0];
    or_f scalar = p->t[1][0];
    if (n <= 1) {
        *q0o = n == 1 ? f_mul(f_mul(scalar, p->t[2][0]), p->t[0][0]) : F_ZERO;
        *qio = F_ZERO;
        return;
    }
    size_t half = n >> 1;
    const or_f *er = p->t[2], *pp = p->t[0];
    or_f q0 = F_ZERO, qi = F_ZERO;
    #pragma omp parallel for reduction(fadd : q0, qi) schedule(static) if (half > PAR_MIN)
    for (size_t i = 0; i < half; i++) {
        q0 = f_add(q0, f_mul(er[i], pp[i]));
        qi = f_add(qi, f_mul(f_sub(er[half + i], er[i]), f_sub(pp[half + i], pp[i])));
    }
    *q0o = f_mul(q0, scalar); *qio = f_mul(qi, scalar);
}

/* GkrProver::round's sums, src/provers/gkr.rs:105-190:
 *   f(x) = add(x) (W_b(x) + W_c(x)) + mult(x) W_b(x) W_c(x)
 * at x = 0, 1, 2 over the pairs (i, i + half), the unpaired tail with an
 * implicit zero hi, then q(inf) = (q(0) + q(2) - 2 q(1)) / 2; a table of at
 * most one entry gives [f, 0]. */
static or_f gkr_term(or_f a, or_f m, or_f wb, or_f wc) {
    return f_add(f_mul(a, f_add(wb, wc)), f_mul(m, f_mul(wb, wc)));
}
static void gkr_compute(const or_prover* p, or_f* q0o, or_f* qio) {
    const size_t n = p->len[0];
    const or_f *A = p->t[0], *M = p->t[1], *WB = p->t[2], *WC = p->t[3];
    if (n <= 1) {
        *q0o = n == 1 ? gkr_term(A[0], M[0], WB[0], WC[0]) : F_ZERO;
        *qio = F_ZERO;
        return;
    }
    const size_t half = next_pow2(n) >> 1, paired = n - half;
    or_f q0 = F_ZERO, q1 = F_ZERO, q2 = F_ZERO;
    for (size_t i = 0; i < paired; i++) {
        const or_f al = A[i], ah = A[i + half], ml = M[i], mh = M[i + half];
        const or_f wbl = WB[i], wbh = WB[i + half], wcl = WC[i], wch = WC[i + half];
        q0 = f_add(q0, gkr_term(al, ml, wbl, wcl));
        q1 = f_add(q1, gkr_term(ah, mh, wbh, wch));
        const or_f a2 = f_sub(f_add(ah, ah), al), m2 = f_sub(f_add(mh, mh), ml);
        const or_f wb2 = f_sub(f_add(wbh, wbh), wbl), wc2 = f_sub(f_add(wch, wch), wcl);
        q2 = f_add(q2, gkr_term(a2, m2, wb2, wc2));
    }
    for (size_t i = paired; i < half && i < n; i++) {
        const or_f al = A[i], ml = M[i], wbl = WB[i], wcl = WC[i];
        q0 = f_add(q0, gkr_term(al, ml, wbl, wcl));
        q2 = f_add(q2, f_sub(f_mul(al, f_add(wbl, wcl)), f_mul(ml, f_mul(wbl, wcl))));
    }
    const or_f inv2 = f_from_u64((OR_P + 1) / 2);
    *q0o = q0;
    *qio = f_mul(f_sub(f_add(q0, q2), f_add(q1, q1)), inv2);
}

/* SumcheckProver::round for every prover (EvalsInfty wire,
 * src/sumcheck_prover.rs:40-59). */
int or_prover_round(or_prover* p, const uint64_t* chal, uint64_t* out, uint64_t* aux) {
    if (p->error) return -1;
    or_f w = chal ? f_load(chal) : F_ZERO;
    or_f r0 = F_ZERO, r1 = F_ZERO;
    switch (p->kind) {
    case OR_ML:   /* src/provers/multilinear.rs:58-67, multilinear_lsb.rs:180-189 */
        if (p->order == OR_MSB) {
            if (chal) fold_msb_pad(p->t[0], &p->len[0], w);
            ml_msb_compute(p->t[0], p->len[0], &r0, &r1);
        } else {
            if (chal) fold_lsb(&p->t[0], &p->len[0], w);
            ml_lsb_compute(p->t[0], p->len[0], &r0, &r1);
        }
        f_store(out, r0);
        break;
    case OR_IP:   /* src/provers/inner_product.rs:61-113, inner_product_lsb.rs:156-164 */
        if (p->order == OR_MSB) {
            if (chal) { fold_msb_pad(p->t[0], &p->len[0], w); fold_msb_pad(p->t[1], &p->len[1], w); }
            ip_msb_compute(p->t[0], p->t[1], p->len[0], &r0, &r1);
        } else {
            if (chal) { fold_lsb(&p->t[0], &p->len[0], w); fold_lsb(&p->t[1], &p->len[1], w); }
            if (ip_lsb_compute(p->t[0], p->t[1], p->len[0], chal == NULL, &r0, &r1)) { p->error = 1; return -1; }
        }
        f_store(out, r0); f_store(out + 3, r1);
        break;
    case OR_COEF: { /* src/provers/coefficient.rs:272-294, coefficient_lsb.rs:180-203 */
        if (chal) coef_reduce(p, w);
        or_f c[4];
        coef_evaluate(p, c);
        int d = p->coef_deg;
        f_store(out, c[0]);
        if (d >= 2) {
            f_store(out + 3, c[d]);
            for (int i = 2; i < d; i++) f_store(out + 3 * i, horner(c, d, f_from_u64((uint64_t)i)));
        }
        r0 = c[0]; r1 = c[1];
        break;
    }
    case OR_EQF: { /* src/provers/eq_factored.rs:249-270 */
        if (chal) {
            size_t prev_var = p->rounds_elapsed - 1;
            fold_msb_pad(p->t[0], &p->len[0], w);
            if (prev_var < p->v_l) fold_msb_pad(p->t[1], &p->len[1], w);
            else fold_msb_pad(p->t[2], &p->len[2], w);
        }
        if (p->rounds_elapsed < p->v_l) eqf_left(p, &r0, &r1);
        else eqf_right(p, &r0, &r1);
        p->rounds_elapsed++;
        f_store(out, r0); f_store(out + 3, r1);
        break;
    }
    case OR_GKR:  /* src/provers/gkr.rs:105-190 */
        if (chal)
            for (int i = 0; i < 4; i++) fold_msb_pad(p->t[i], &p->len[i], w);
        gkr_compute(p, &r0, &r1);
        f_store(out, r0); f_store(out + 3, r1);
        break;
    default: return -1;
    }
    if (aux) { f_store(aux, r0); f_store(aux + 3, r1); }
    return 0;
}

void or_prover_finalize(or_prover* p, const uint64_t* chal) {
    or_f w = f_load(chal);
    switch (p->kind) {
    case OR_ML:
        if (p->order == OR_MSB) fold_msb_pad(p->t[0], &p->len[0], w);
        else fold_lsb(&p->t[0], &p->len[0], w);
        break;
    case OR_IP:
        for (int i = 0; i < 2; i++) {
            if (p->order == OR_MSB) fold_msb_pad(p->t[i], &p->len[i], w);
            else fold_lsb(&p->t[i], &p->len[i], w);
        }
        break;
    case OR_COEF:
        coef_reduce(p, w);
        break;
    case OR_GKR:   /* src/provers/gkr.rs:193-198 */
        for (int i = 0; i < 4; i++) fold_msb_pad(p->t[i], &p->len[i], w);
        break;
    case OR_EQF: { /* src/provers/eq_factored.rs:272-280: last_var = v - 1 (wrapping) */
        size_t last_var = p->v - 1;
        fold_msb_pad(p->t[0], &p->len[0], w);
        if (last_var < p->v_l) fold_msb_pad(p->t[1], &p->len[1], w);
        else fold_msb_pad(p->t[2], &p->len[2], w);
        break;
    }
    }
}

void or_prover_final_value(const or_prover* p, uint64_t* out) {
    or_f r = F_ZERO;
    switch (p->kind) {
    case OR_ML:   /* src/provers/multilinear.rs:74-79 */
        if (p->len[0] == 1) r = p->t[0][0];
        break;
    case OR_IP:   /* src/provers/inner_product.rs:120-126 */
        if (p->len[0] == 1) r = f_mul(p->t[0][0], p->t[1][0]);
        break;
    case OR_COEF: { /* src/provers/coefficient.rs:300-329, coefficient_lsb.rs:209-236 */
        if (p->ntab == 1 && p->len[0] == 1) { r = p->t[0][0]; break; }
        or_f lo[3], hi[3];
        for (int i = 0; i < p->ntab; i++) {
            lo[i] = p->len[i] == 1 ? p->t[i][0] : F_ZERO;
            hi[i] = F_ZERO;
        }
        or_f c[4] = {F_ZERO, F_ZERO, F_ZERO, F_ZERO};
        product_accumulate(c, p->ntab, lo, hi);
        r = f_add(horner(c, p->coef_deg, F_ZERO), horner(c, p->coef_deg, F_ONE));
        break;
    }
    case OR_EQF:  /* src/provers/eq_factored.rs:282-288 */
        if (p->len[0] == 1) r = f_mul(f_mul(p->t[0][0], p->t[1][0]), p->t[2][0]);
        break;
    case OR_GKR:  /* src/provers/gkr.rs:200-208 */
        if (p->len[0] == 1) r = gkr_term(p->t[0][0], p->t[1][0], p->t[2][0], p->t[3][0]);
        break;
    }
    f_store(out, r);
}

/* ========================================================================== */
/* Runner, src/runner.rs:29-69 (legacy runners: src/multilinear_sumcheck.rs:    */
/* 265-319 sends (s0, s1); src/inner_product_sumcheck.rs:507-565 sends          */
/* (c0, c2)).                                                                   */
/* ========================================================================== */
int or_sumcheck(or_prover* p, size_t num_rounds, or_transcript* t,
                const uint8_t* hook, size_t hook_len, int legacy,
                uint64_t* round_polys, uint64_t* challenges, uint64_t* final_value) {
    int d = or_prover_degree(p);
    int nsend = legacy ? 2 : d;
    uint64_t prev[3];
    int have = 0;
    for (size_t r = 0; r < num_rounds; r++) {
        uint64_t out[12], aux[6];
        if (or_prover_round(p, have ? prev : NULL, out, aux)) return -1;
        const uint64_t* msg = legacy ? aux : out;
        for (int i = 0; i < nsend; i++) {
            or_transcript_send(t, msg + 3 * i);
            if (round_polys) memcpy(round_polys + 3 * ((size_t)r * nsend + i), msg + 3 * i, 24);
        }
        if (hook_len) or_transcript_absorb(t, hook, hook_len);
        or_transcript_challenge(t, prev);
        have = 1;
        if (challenges) memcpy(challenges + 3 * r, prev, 24);
    }
    if (have) or_prover_finalize(p, prev);
    if (final_value) or_prover_final_value(p, final_value);
    return 0;
}

/* Barycentric weight, src/verifier.rs:187-200. */
static uint64_t bary_weight(size_t i, size_t d) {
    uint64_t w = 1;
    for (size_t j = 0; j < d; j++) {
        if (j == i) continue;
        long long diff = (long long)i - (long long)j;
        uint64_t f = diff > 0 ? (uint64_t)diff : or_fp_sub(0, (uint64_t)(-diff));
        w = or_fp_mul(w, f);
    }
    return w;
}
/* evaluate_from_evals, src/verifier.rs:146-184. */
static or_f eval_from_evals(const or_f* ev, size_t d, or_f r) {
    if (d == 0) return F_ZERO;
    if (d == 1) return ev[0];
    if (d == 2) return f_add(ev[0], f_mul(r, f_sub(ev[1], ev[0])));
    or_f rm[8], pre[9], suf[9];
    for (size_t j = 0; j < d; j++) rm[j] = f_sub(r, f_from_u64(j));
    pre[0] = F_ONE;
    for (size_t i = 0; i < d; i++) pre[i + 1] = f_mul(pre[i], rm[i]);
    suf[d] = F_ONE;
    for (size_t i = d; i-- > 0;) suf[i] = f_mul(suf[i + 1], rm[i]);
    or_f res = F_ZERO;
    for (size_t i = 0; i < d; i++) {
        or_f inv = {{or_fp_inv(bary_weight(i, d)), 0, 0}};
        res = f_add(res, f_mul(f_mul(ev[i], f_mul(pre[i], suf[i + 1])), inv));
    }
    return res;
}
/* sumcheck_verify, src/verifier.rs:61-139.  The transcript receive absorbs
 * the proof's value exactly as the prover's send did. */
int or_verify(const uint64_t* claimed_sum, size_t degree, size_t num_rounds,
              or_transcript* t, const uint8_t* hook, size_t hook_len,
              const uint64_t* round_polys, uint64_t* challenges, uint64_t* final_claim) {
    or_f claim = f_load(claimed_sum);
    size_t d = degree, n_wire = d > 1 ? d : 1;
    for (size_t round = 0; round < num_rounds; round++) {
        or_f recv[8];
        for (size_t i = 0; i < n_wire; i++) {
            const uint64_t* v = round_polys + 3 * (round * n_wire + i);
            or_transcript_send(t, v);
            recv[i] = f_load(v);
        }
        or_f h0 = recv[0], h1 = f_sub(claim, h0);
        if (hook_len) or_transcript_absorb(t, hook, hook_len);
        uint64_t rr[3];
        or_transcript_challenge(t, rr);
        or_f r = f_load(rr);
        if (challenges) memcpy(challenges + 3 * round, rr, 24);
        if (d == 0) { claim = h0; continue; }
        or_f h_inf = d >= 2 ? recv[1] : f_sub(h1, h0);
        or_f q[8];
        q[0] = h0;
        q[1] = f_sub(h1, h_inf);
        for (size_t i = 2; i < d; i++) {
            or_f idd = F_ONE, fi = f_from_u64(i);
            for (size_t k = 0; k < d; k++) idd = f_mul(idd, fi);
            q[i] = f_sub(recv[i], f_mul(h_inf, idd));
        }
        or_f qr = eval_from_evals(q, d, r);
        or_f rd = F_ONE;
        for (size_t k = 0; k < d; k++) rd = f_mul(rd, r);
        claim = f_add(qr, f_mul(h_inf, rd));
    }
    f_store(final_claim, claim);
    return 0;
}

/* Independent MLE evaluation (MSB halving), tests/canonical_api.rs:22-34. */
void or_mle_eval_msb(const uint64_t* table, size_t len, const uint64_t* point, size_t v, uint64_t* out) {
    or_f* cur = load_table(table, len, 3);
    size_t n = len;
    for (size_t j = 0; j < v; j++) {
        or_f r = f_load(point + 3 * j);
        size_t half = n / 2;
        for (size_t i = 0; i < half; i++) cur[i] = f_add(cur[i], f_mul(f_sub(cur[i + half], cur[i]), r));
        n = half;
    }
    f_store(out, n ? cur[0] : F_ZERO);
    free(cur);
}

/* protogalaxy::fold (src/folding.rs:14-75) as a release build runs it:
 * level k pairs polynomial 2i with 2i+1 (an odd last one is dropped) into
 * p[2i] + (a_k + b_k X)(p[2i+1] - p[2i]), each level raising the degree
 * bound by one; levels after a single polynomial remains change nothing.
 * polys: n rows of `width` coefficients (ncomp = 1 or 3 words each,
 * ascending degree, zero-padded); pairs: levels x (a, b), 3 words each.  out: width + levels coefficients;
 * *out_len = the length of the result with trailing zeros trimmed -- at
 * least 1 for n >= 2 (to_dense_poly, src/poly_ops.rs:159-166), 0 for the
 * zero polynomial at n = 0, the input's own trimmed length at n = 1. */
void or_pg_fold(const uint64_t* pairs, size_t levels, const uint64_t* polys, size_t n, size_t width, int ncomp,
                uint64_t* out, size_t* out_len) {
    const size_t slot = width + levels;
    size_t len = 0;
    for (size_t j = 0; j < slot; j++) f_store(out + 3 * j, F_ZERO);
    if (n == 0) { *out_len = 0; return; }
    or_f* buf = (or_f*)calloc(n * (slot ? slot : 1), sizeof(or_f));
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < width; j++) {
            const uint64_t* src = polys + (size_t)ncomp * (i * width + j);
            or_f x = F_ZERO;
            for (int c = 0; c < ncomp; c++) x.c[c] = src[c];
            buf[i * slot + j] = x;
        }
    size_t count = n, w = width;
    if (n >= 2) {
        for (size_t k = 0; k < levels && count >= 2; k++) {
            const or_f a = f_load(pairs + 6 * k), b = f_load(pairs + 6 * k + 3);
            const size_t half = count / 2;
            or_f* nxt = (or_f*)calloc(half * slot, sizeof(or_f));
            #pragma omp parallel for schedule(static) if (half * w > PAR_MIN)
            for (size_t i = 0; i < half; i++) {
                const or_f* p0 = buf + 2 * i * slot;
                const or_f* p1 = buf + (2 * i + 1) * slot;
                or_f prev = F_ZERO;
                for (size_t j = 0; j <= w; j++) {
                    const or_f d = j < w ? f_sub(p1[j], p0[j]) : F_ZERO;
                    const or_f base = j < w ? p0[j] : F_ZERO;
                    nxt[i * slot + j] = f_add(base, f_add(f_mul(a, d), f_mul(b, prev)));
                    prev = d;
                }
            }
            free(buf);
            buf = nxt;
            count = half;
            w++;
        }
        len = w;
        while (len > 1 && f_eq(buf[len - 1], F_ZERO)) len--;
    } else {
        len = width;
        while (len > 0 && f_eq(buf[len - 1], F_ZERO)) len--;
    }
    for (size_t j = 0; j < len; j++) f_store(out + 3 * j, buf[j]);
    *out_len = len;
    free(buf);
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int or_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
