/*
 * effsc_oracle.h -- CPU oracle for the sumcheck fold+evaluate path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * crate `effsc` (compsec-epfl/efficient-sumcheck) provers, runner, verifier and
 * field arithmetic.  Only the test suite, the smoke check and the CPU-baseline
 * leg of the benchmark load it, and only as the checker.  The GPU library never
 * links or calls it.
 *
 * Parity status: the reference is Rust and cannot be built in this environment
 * (no cargo/rustc, arkworks/spongefish not vendored), and its own tests hold no
 * golden values -- they pin behaviour through properties (fused == unfused,
 * MLE evaluation at the challenges, verifier acceptance, split == full,
 * EqFactored == InnerProduct(eq table), Coefficient(deg 1) == Multilinear).
 * This oracle is pinned against those properties, against the Montgomery
 * known-answer constants in src/tests/fields.rs:62-63, and against an
 * independent big-integer Python restatement; see tests/test_oracle.py.
 *
 * Representation: every element of the prover field F is held as an Fp3
 * triple (c0, c1, c2) of canonical Goldilocks values; base-field elements are
 * the embedded triples (x, 0, 0).  Fp3 = Fp[X]/(X^3 - W) with W the canonical
 * value of the crate's F64Ext3 non-residue `F64::from_raw(7)` (a Montgomery
 * raw value), i.e. W = 7 * 2^-64 mod p = 0xFFFFFFF800000001
 * (src/tests/fields.rs:73-100).
 */
#ifndef EFFSC_ORACLE_H
#define EFFSC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_P   0xFFFFFFFF00000001ULL
#define OR_EPS 0x00000000FFFFFFFFULL
#define OR_W   0xFFFFFFF800000001ULL

typedef struct { uint64_t c[3]; } or_f;

/* ---- field ---------------------------------------------------------------- */
uint64_t or_fp_add(uint64_t a, uint64_t b);
uint64_t or_fp_sub(uint64_t a, uint64_t b);
uint64_t or_fp_mul(uint64_t a, uint64_t b);
uint64_t or_fp_inv(uint64_t a);
uint64_t or_fp_to_mont(uint64_t a);
uint64_t or_fp_from_mont(uint64_t a);
void or_f3_mul(const uint64_t* a, const uint64_t* b, uint64_t* out);

/* ---- seeded generator ------------------------------------------------------ */
uint64_t or_splitmix64_mix(uint64_t z);
uint64_t or_table_seed(uint64_t seed, uint64_t table);
uint64_t or_gen_element(uint64_t seed, uint64_t i);
void or_gen_table(uint64_t seed, uint64_t n, uint64_t* out);

/* ---- transcripts ----------------------------------------------------------- */
enum { OR_T_KECCAK = 0, OR_T_TEST = 1 };
typedef struct {
    int kind;            /* OR_T_KECCAK or OR_T_TEST                      */
    int deg;             /* 1: F = Fp, 3: F = Fp3                         */
    uint64_t st[25];     /* Keccak-f[1600] state                          */
    uint32_t pos;        /* byte position inside the rate                 */
    uint32_t squeezing;  /* 0 absorbing, 1 squeezing                      */
    uint64_t sm;         /* SplitMix64 state for the test transcript      */
} or_transcript;

void or_keccak_f1600(uint64_t* st);
void or_transcript_init_keccak(or_transcript* t, int deg, const uint8_t* label, size_t len);
void or_transcript_init_test(or_transcript* t, int deg, uint64_t seed);
void or_transcript_absorb(or_transcript* t, const uint8_t* data, size_t len);
void or_transcript_squeeze(or_transcript* t, uint8_t* out, size_t len);
void or_transcript_send(or_transcript* t, const uint64_t* v);
void or_transcript_challenge(or_transcript* t, uint64_t* out);
size_t or_transcript_size(void);

/* ---- provers --------------------------------------------------------------- */
enum { OR_ML = 0, OR_IP = 1, OR_COEF = 2, OR_EQF = 3, OR_GKR = 4 };
enum { OR_MSB = 0, OR_LSB = 1 };

typedef struct {
    int kind, order, deg;
    int ntab;            /* tables in use                                 */
    size_t len[4];
    or_f* t[4];          /* EQF: t[0] = p, t[1] = eq_l, t[2] = eq_r       */
    int coef_deg;        /* COEF: degree of the product evaluator (ntab)  */
                         /* GKR: t = add, mult, w_b, w_c (broadcast)      */
    size_t v, v_l, rounds_elapsed;
    int error;           /* set when the reference would panic            */
} or_prover;

/* Tables are given as `ncomp` u64 per element (1: base, 3: Fp3 AoS). */
or_prover* or_prover_new(int kind, int order, int deg, int ntab,
                         const uint64_t* const* tables, const size_t* lens, int ncomp);
or_prover* or_eqf_new(int deg, const uint64_t* w, size_t v, const uint64_t* p, size_t plen, int ncomp);
/* GkrProver::new (src/provers/gkr.rs:61-82): add, mult of n*n elements, w of
 * n elements; the witness is expanded into the broadcast tables w_b, w_c. */
or_prover* or_gkr_new(int deg, const uint64_t* add, const uint64_t* mult, const uint64_t* w, size_t n, int ncomp);
/* GkrProver::claimed_w_values (src/provers/gkr.rs:87-93): out = 2 elements. */
void or_gkr_claimed_w_values(const or_prover* p, uint64_t* out);
void or_prover_free(or_prover* p);
int  or_prover_degree(const or_prover* p);
/* out: `degree` elements (wire, EvalsInfty).  aux (optional): the two raw
 * per-round values (ML: s0,s1; IP: q0,qinf) used by the legacy runners. */
int  or_prover_round(or_prover* p, const uint64_t* chal, uint64_t* out, uint64_t* aux);
void or_prover_finalize(or_prover* p, const uint64_t* chal);
void or_prover_final_value(const or_prover* p, uint64_t* out);
size_t or_prover_table_len(const or_prover* p, int i);
void or_prover_read_table(const or_prover* p, int i, uint64_t* out /* 3 per element */);

/* ---- runner / verifier ------------------------------------------------------ */
/* round_polys: num_rounds * degree elements (3 u64 each); challenges:
 * num_rounds elements; final_value: 1 element.  hook: `hook_len` bytes
 * absorbed after each round's messages (NULL / 0 for the no-op hook).
 * legacy != 0 sends the aux pair instead of the EvalsInfty wire. */
int or_sumcheck(or_prover* p, size_t num_rounds, or_transcript* t,
                const uint8_t* hook, size_t hook_len, int legacy,
                uint64_t* round_polys, uint64_t* challenges, uint64_t* final_value);
int or_verify(const uint64_t* claimed_sum, size_t degree, size_t num_rounds,
              or_transcript* t, const uint8_t* hook, size_t hook_len,
              const uint64_t* round_polys, uint64_t* challenges, uint64_t* final_claim);

void or_build_eq_table(const uint64_t* w, size_t v, uint64_t* out /* 3 * 2^v */);
void or_mle_eval_msb(const uint64_t* table, size_t len, const uint64_t* point, size_t v, uint64_t* out);

/* protogalaxy::fold (src/folding.rs:14-75), release-build semantics: n
 * polynomials of `width` coefficients (ncomp words each, zero-padded), `levels`
 * pairs (a, b); out holds width + levels coefficients, *out_len the trimmed
 * length (>= 1 for n >= 2, 0 for n = 0). */
void or_pg_fold(const uint64_t* pairs, size_t levels, const uint64_t* polys, size_t n, size_t width, int ncomp,
                uint64_t* out, size_t* out_len);

void or_set_threads(int n);
int  or_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
