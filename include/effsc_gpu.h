/*
 * effsc_gpu.h -- C ABI of the GB300 sumcheck prover.
 *
 * The entry points are what a Rust binding of the crate `effsc`
 * (compsec-epfl/efficient-sumcheck) needs to keep its prover API as a drop-in
 * while the fold+evaluate rounds run on one sm_103a GPU.  Each function names
 * the reference item it stands in for (paths relative to that crate's root).
 *
 * Conventions
 *  - Every function returns an effsc_status; on failure
 *    effsc_last_error() returns a thread-local message.  EFFSC_PANIC marks the
 *    cases where the reference panics (e.g. unequal table lengths).
 *  - Field elements are uint64_t words.  A prover's field F is Fp
 *    (EFFSC_FP, 1 word per element) or the cubic extension F64Ext3
 *    (EFFSC_FP3, 3 words [c0, c1, c2] per element, the layout of arkworks'
 *    CubicExtField).  Tables may also be passed as base-field words
 *    (ncomp = 1) for an Fp3 prover: they are the embedded elements (x, 0, 0),
 *    exactly what the reference receives as "lifted" tables.
 *  - repr selects the word encoding at the boundary: EFFSC_CANONICAL
 *    (0 <= x < p) or EFFSC_MONTGOMERY (arkworks' x * 2^64 mod p, so that
 *    `&[F]` reinterpreted as `&[u64]` can be passed without a copy,
 *    reference src/field.rs:314-375).  The device computes in canonical form.
 *  - Handles are not re-entrant: one thread at a time per handle.
 *  - Host pointers are plain host memory (pageable or pinned).
 */
#ifndef EFFSC_GPU_H
#define EFFSC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    EFFSC_OK = 0,
    EFFSC_INVALID_ARG = 1,
    EFFSC_OOM = 2,
    EFFSC_CUDA_ERROR = 3,
    EFFSC_TIMEOUT = 4,
    EFFSC_UNSUPPORTED = 5,
    EFFSC_PANIC = 6
} effsc_status;

typedef enum { EFFSC_ML = 0, EFFSC_IP = 1, EFFSC_COEF = 2, EFFSC_EQF = 3, EFFSC_GKR = 4 } effsc_kind;
typedef enum { EFFSC_MSB = 0, EFFSC_LSB = 1 } effsc_order;
typedef enum { EFFSC_FP = 1, EFFSC_FP3 = 3 } effsc_field;
typedef enum { EFFSC_CANONICAL = 0, EFFSC_MONTGOMERY = 1 } effsc_repr;
typedef enum { EFFSC_T_KECCAK = 0, EFFSC_T_TEST = 1 } effsc_transcript_kind;

typedef struct effsc_ctx effsc_ctx;
typedef struct effsc_prover effsc_prover;
typedef struct effsc_transcript effsc_transcript;

/* ---- errors / library -------------------------------------------------- */
const char* effsc_last_error(void);
const char* effsc_status_str(int status);
/* Number of kernel launches issued by this thread since the last reset. */
uint64_t effsc_launch_count(void);
void effsc_launch_count_reset(void);

/* Measurement (no reference counterpart).  While enabled on a thread, every
 * kernel that thread launches outside a CUDA graph is bracketed by CUDA events
 * on its stream and recorded with its algorithmic bytes (table words it must
 * read plus words it writes).  effsc_profile_get waits for record i. */
int effsc_profile_enable(int on);
size_t effsc_profile_count(void);
int effsc_profile_get(size_t i, char* name, size_t name_cap, double* ms, uint64_t* bytes);
void effsc_profile_clear(void);

/* ---- context: one GPU and one CUDA stream -------------------------------- */
/* No reference counterpart (the crate is CPU-only); every prover, transcript
 * upload and batch runs on the context's stream. */
int effsc_ctx_create(int device, effsc_ctx** out);
int effsc_ctx_destroy(effsc_ctx* ctx);
/* Use an external cudaStream_t (NULL restores the context's own stream). */
int effsc_ctx_set_stream(effsc_ctx* ctx, void* cuda_stream);
int effsc_ctx_synchronize(effsc_ctx* ctx);

/* ---- provers --------------------------------------------------------------
 * kind/order select the reference prover:
 *   EFFSC_ML  MSB: MultilinearProver::new(evals)      src/provers/multilinear.rs:30-33
 *   EFFSC_ML  LSB: MultilinearProverLSB::new(evals)   src/provers/multilinear_lsb.rs:31-35
 *   EFFSC_IP  MSB: InnerProductProver::new(a, b)      src/provers/inner_product.rs:33-36
 *   EFFSC_IP  LSB: InnerProductProverLSB::new(a, b)   src/provers/inner_product_lsb.rs:31-34
 *   EFFSC_COEF MSB/LSB: CoefficientProver[LSB]::new(&E, vec![], pairwise)
 *                   src/provers/coefficient.rs:28-40, coefficient_lsb.rs:51-66,
 *                   with E the device product evaluator of degree n_tables
 *                   (1..3): accumulate_pair adds the coefficients of
 *                   prod_i (lo_i + x (hi_i - lo_i)) -- TripleProductEval
 *                   (tests/adversarial_verifier.rs:444-466) for n_tables = 3.
 * tables[i] has lens[i] elements of ncomp[i] words (1: base field, 3: Fp3).
 * IP with lens[0] != lens[1] returns EFFSC_PANIC like the reference's assert.
 * The input tables are copied to the device; the prover owns the copies. */
int effsc_prover_create(effsc_ctx* ctx, int kind, int order, int field, int repr,
                        int n_tables, const uint64_t* const* tables, const size_t* lens,
                        const int* ncomp, effsc_prover** out);
/* EqFactoredProver::new(w, p_evals), src/provers/eq_factored.rs:90-114.
 * w: num_vars elements of `field`; p: p_len <= 2^num_vars elements of
 * p_ncomp words (zero-padded to 2^num_vars; longer is EFFSC_PANIC). */
int effsc_eqf_create(effsc_ctx* ctx, int field, int repr, const uint64_t* w, size_t num_vars,
                     const uint64_t* p, size_t p_len, int p_ncomp, effsc_prover** out);
/* The constructors above over tables left in HOST memory and read in place by
 * the kernels (no bulk copy; for tables larger than HBM: only the folded
 * tables are allocated on the device).  Layout as effsc_prover_create_device.
 * Pinned or registered memory always works; plain pageable memory (including
 * a memory-mapped file) works when the GPU reads host page tables
 * (cudaDevAttrPageableMemoryAccess), else EFFSC_UNSUPPORTED.  The memory must
 * stay valid and unchanged while the prover exists (its input tables are
 * never written).  No reference counterpart (the crate's FileStream /
 * MemoryStream, src/streams/, feed provers from memory or mmap). */
int effsc_prover_create_host(effsc_ctx* ctx, int kind, int order, int field, int n_tables,
                             const uint64_t* const* host_tables, const size_t* lens, const int* ncomp,
                             effsc_prover** out);

/* reorder_vec_msb, src/streams/memory/core.rs:20-47: dst[i] = src[bit_reverse(i)]
 * over n (a power of two, else EFFSC_PANIC as the reference asserts) elements
 * of ncomp words; src and dst in host or device memory. */
int effsc_reorder_msb(effsc_ctx* ctx, const uint64_t* src, size_t n, int ncomp, uint64_t* dst);
/* multivariate_claim (n_tables = 1) and multivariate_product_claim
 * (src/streams/stream.rs:3-40): out = sum over i < n of prod_t tables[t][i],
 * `field` words; tables canonical with ncomp words per element (AoS), in host
 * or device memory, read in place; 1..4 tables. */
int effsc_stream_claim(effsc_ctx* ctx, int field, int n_tables, const uint64_t* const* tables, size_t n, int ncomp,
                       uint64_t* out);

/* GkrProver::new(add_evals, mult_evals, w_evals), src/provers/gkr.rs:61-82:
 * add and mult hold n * n elements, w holds n (a power of two, n <= 2^17),
 * `ncomp` u64 per element, `repr` as above.  The prover runs 2 log2(n)
 * rounds of degree 2; its tables are add, mult and the witness kept as two
 * n-element tables W_b (0..n-1 over b) and W_c (over c) instead of the
 * reference's broadcast n*n tables (same values).  The reference's
 * constructor asserts the lengths; here the caller passes n. */
int effsc_gkr_create(effsc_ctx* ctx, int field, int repr, const uint64_t* add, const uint64_t* mult, const uint64_t* w,
                     size_t n, int ncomp, effsc_prover** out);
/* GkrProver::claimed_w_values, src/provers/gkr.rs:87-93: (W(b*), W(c*)) once
 * all 2 log2(n) variables are bound, else zeros; out = 2 elements. */
int effsc_gkr_claimed_w_values(effsc_prover* p, uint64_t* out);
/* CoefficientProver::new / CoefficientProverLSB::new (src/provers/coefficient.rs:28-40,
 * coefficient_lsb.rs:37-99) with a declarative RoundPolyEvaluator
 * (src/coefficient_sumcheck.rs:50-76): per pair of rows, every term adds
 *   k * (product of its factors)
 * into coefficient `coeff` of the round polynomial.  A factor names the even
 * (lo) or odd (hi) element of a column: factor = column * 2 + (0 | 1), the
 * columns being the pairwise tables (0 .. n_pairwise-1) and then the columns
 * of each tablewise table in order (a tablewise table of width w is len rows
 * of w elements, row-major, tw_ncomp words each; its row pair is its columns'
 * element pairs).  Every table has len entries (rows).  Degree 0..3, at most
 * 4 columns, 16 terms, 4 factors per term; k is one field element in the
 * prover's representation.  The prover is then driven like the others
 * (effsc_prover_round, effsc_prove, finalize, final_value, read_table of
 * column i); out_aux of a round holds (c0, c1).  This covers evaluators whose
 * accumulate_pair is a sum of constant multiples of products of pair
 * elements -- e.g. the reference's Degree1, Degree2, Mixed and InnerProduct
 * test evaluators (src/coefficient_sumcheck.rs:379-430); a Rust closure of
 * any other shape cannot run on the device. */
typedef struct {
    uint32_t coeff;        /* coefficient index, 0..degree */
    uint32_t n_factors;    /* 0..4; 0 adds k once per pair */
    uint32_t factors[4];   /* column * 2 + (0: even element, 1: odd element) */
    uint64_t k[3];         /* the constant, `field` words */
} effsc_term;
int effsc_coef_expr_create(effsc_ctx* ctx, int order, int field, int repr, int degree, int n_pairwise,
                           const uint64_t* const* pairwise, const int* pw_ncomp, int n_tablewise,
                           const uint64_t* const* tablewise, const size_t* tw_widths, const int* tw_ncomp,
                           size_t len, const effsc_term* terms, size_t n_terms, effsc_prover** out);
/* Same constructors with the tables already in device memory (canonical,
 * structure-of-arrays: c0 of every element, then c1, then c2 when ncomp = 3);
 * the prover copies nothing and does not take ownership: the caller keeps the
 * buffers alive and unchanged until the prover is destroyed.  Rounds never
 * write to these buffers, so effsc_prover_reset() can rerun the proof. */
int effsc_prover_create_device(effsc_ctx* ctx, int kind, int order, int field,
                               int n_tables, const uint64_t* const* dev_tables, const size_t* lens,
                               const int* ncomp, effsc_prover** out);
int effsc_prover_destroy(effsc_prover* p);

/* SumcheckProver::degree, src/sumcheck_prover.rs:36-71. */
int effsc_prover_degree(const effsc_prover* p);
/* SumcheckProver::round, src/sumcheck_prover.rs:40-59: challenge == NULL is
 * round(None) (round 0); otherwise fold with *challenge and compute the next
 * round polynomial.  out_evals receives degree() elements in the EvalsInfty
 * wire format [h(0)] (d = 1) or [h(0), h(inf), h(2), ..., h(d-1)].  out_aux
 * (optional, 2 elements) receives the raw per-round pair the legacy runners
 * send: (s0, s1) for ML (src/multilinear_sumcheck.rs:9-14), (c0, c2) for IP
 * (src/inner_product_sumcheck.rs:11-16), (c0, c1) for COEF. */
int effsc_prover_round(effsc_prover* p, const uint64_t* challenge, uint64_t* out_evals, uint64_t* out_aux);
/* SumcheckProver::finalize, src/sumcheck_prover.rs:61-66. */
int effsc_prover_finalize(effsc_prover* p, const uint64_t* challenge);
/* SumcheckProver::final_value, src/sumcheck_prover.rs:68-70. */
int effsc_prover_final_value(effsc_prover* p, uint64_t* out);
/* Post-state accessors: InnerProductProver::evaluations / MultilinearProver::evals
 * / CoefficientProver::pairwise / EqFactoredProver tables (p, eq_l, eq_r).
 * Writes table_len() elements of `field` words each (AoS). */
int effsc_prover_table_len(const effsc_prover* p, int table, size_t* out_len);
int effsc_prover_read_table(effsc_prover* p, int table, uint64_t* out);
/* effsc_prove only (no reference counterpart; a tuning knob): once an MSB
 * Multilinear / InnerProduct prover's power-of-two tables are at most
 * max_len long, the remaining rounds run in one launch with the tables in
 * shared memory: one thread block, or (Multilinear, tables up to 16 times
 * one block's capacity, entered mid-proof) a thread-block cluster that hands
 * over to one block.  A GkrProver's rounds move into one block once add,
 * mult, W_b and W_c fit in shared memory together and add is at most max_len
 * long.  Default SIZE_MAX: as long as shared memory allows; 0 disables.
 * Proofs are identical. */
int effsc_prover_set_tail(effsc_prover* p, size_t max_len);
/* effsc_prove only (no reference counterpart; a tuning knob): for an
 * InnerProduct prover (MSB or LSB) over Fp3 challenges or an MSB Multilinear
 * prover with power-of-two base tables, and for a GkrProver with |w| >= 8
 * over base add, mult and w, fused = 1 computes rounds 0-2 in two passes over
 * the base tables (round 1 from sums gathered during round 0; round 2 folds
 * with both challenges).  fused = 2 (the default) does the same and, for an
 * InnerProduct prover with base tables of 2^14 entries or more and at least
 * 4 rounds, computes rounds 0-3 in two passes instead (rounds 0-2 from 26
 * interpolation sums of one pass; round 3 folds with three challenges).
 * For a CoefficientProver with the degree-3 product evaluator over three
 * tables of 2^12 entries or more (table 0 in Fp or Fp3, tables 1-2 in Fp),
 * fused >= 1 computes rounds 0-2 in two passes (rounds 0 and 1 from 15
 * triple-product sums of one pass; round 2 folds with both challenges).
 * 0 runs one pass per round.  Proofs are identical. */
int effsc_prover_set_first_rounds(effsc_prover* p, int fused);
/* effsc_prove only (no reference counterpart; a tuning knob): for an
 * InnerProduct prover over Fp3 challenges, consecutive rounds whose tables
 * hold at most max_len entries (after the first fold, down to the tail) run
 * in one cooperative launch with a grid barrier between rounds, the last
 * block to arrive running the transcript step.  Default 0 (off); 2^21 covers
 * the rounds after the two-pass start of a 2^26 proof.  Proofs are identical. */
int effsc_prover_set_persistent(effsc_prover* p, size_t max_len);

/* Restore the state right after construction (the input tables are never
 * written by the rounds), so a proof can be recomputed without re-upload. */
int effsc_prover_reset(effsc_prover* p);

/* The whole protocol on the device: runner::sumcheck (src/runner.rs:29-69)
 * with the device transcript -- per round the wire values and `hook` bytes
 * (hook_len may be 0) are absorbed into `t` and the next challenge squeezed on
 * the GPU.  `t` must be an EFFSC_T_KECCAK transcript of the prover's field;
 * its state is uploaded first and written back at the end, so host-side
 * sends/challenges can be interleaved with device proofs (partial runs).
 * Outputs (host, may be NULL): round_polys (num_rounds * degree elements),
 * challenges (num_rounds elements), final_value (1 element).
 * use_graph != 0 captures the launches in a CUDA graph and replays it; the
 * graph is cached per (prover, num_rounds, hook_len) and reused by later
 * calls after effsc_prover_reset(). */
int effsc_prove(effsc_prover* p, size_t num_rounds, effsc_transcript* t,
                const uint8_t* hook, size_t hook_len, int use_graph,
                uint64_t* round_polys, uint64_t* challenges, uint64_t* final_value);

/* ---- transcripts ---------------------------------------------------------
 * ProverTranscript / VerifierTranscript (src/transcript/transcript.rs:11-43).
 * EFFSC_T_KECCAK: the project's Fiat-Shamir transcript (Keccak-f[1600]
 *   duplex, 136-byte rate; label absorbed as 8-byte LE length + bytes;
 *   elements absorbed as 8 LE bytes per component; a challenge component is
 *   16 squeezed LE bytes mod p).  The crate's default spongefish transcript
 *   (src/transcript/spongefish.rs:17-44) is not reproduced.
 * EFFSC_T_TEST: SanityTranscript semantics (src/transcript/sanity.rs:12-55):
 *   sends are no-ops, challenge = F::from_u64(next_u64()) from a SplitMix64
 *   stream seeded with `seed`. */
int effsc_transcript_create(int kind, int field, int repr, const uint8_t* label, size_t label_len,
                            uint64_t seed, effsc_transcript** out);
int effsc_transcript_destroy(effsc_transcript* t);
int effsc_transcript_clone(const effsc_transcript* t, effsc_transcript** out);
int effsc_transcript_absorb(effsc_transcript* t, const uint8_t* bytes, size_t len);
int effsc_transcript_squeeze(effsc_transcript* t, uint8_t* out, size_t len);
int effsc_transcript_send(effsc_transcript* t, const uint64_t* value);
int effsc_transcript_challenge(effsc_transcript* t, uint64_t* out);

/* ---- verifier --------------------------------------------------------------
 * sumcheck_verify, src/verifier.rs:61-139, on the host: receives degree
 * values per round from round_polys (absorbing them into t), applies the hook
 * bytes, squeezes the challenge and reduces the claim.  The oracle check
 * final_claim == final_value stays with the caller, as in the reference. */
int effsc_verify(int field, int repr, const uint64_t* claimed_sum, size_t degree, size_t num_rounds,
                 effsc_transcript* t, const uint8_t* hook, size_t hook_len,
                 const uint64_t* round_polys, uint64_t* challenges, uint64_t* final_claim);

/* ---- standalone fold -------------------------------------------------------
 * effsc::fold (src/fold.rs:14 -> src/multilinear_sumcheck.rs:132-178):
 * values[k] + weight * (values[k + L/2] - values[k]) with implicit zero
 * padding to the next power of two; *out_len = next_pow2(len)/2 (len <= 1:
 * unchanged).  values: len elements of ncomp words; out: *out_len elements of
 * `field` words. */
int effsc_fold(effsc_ctx* ctx, int field, int repr, const uint64_t* values, size_t len, int ncomp,
               const uint64_t* weight, uint64_t* out, size_t* out_len);

/* ---- round polynomial of a multilinear table (the WHIR-facing helpers) -----
 * compute_sumcheck_polynomial (src/multilinear_sumcheck.rs:86-124):
 * out_s0_s1 = (s0, s1) of values with implicit zero padding to the next
 * power of two -- s0 = sum of the low half (plus the unpaired tail), s1 = sum
 * of the high half; (v[0], 0) for one element, (0, 0) for none.  2 elements
 * of `field` words. */
int effsc_compute_sumcheck_polynomial(effsc_ctx* ctx, int field, int repr, const uint64_t* values, size_t len,
                                      int ncomp, uint64_t* out_s0_s1);
/* fused_fold_and_compute_polynomial (src/multilinear_sumcheck.rs:189-254):
 * folds values by weight exactly as effsc_fold does (*out_len elements of
 * `field` words to out) and returns the folded table's (s0, s1) as
 * effsc_compute_sumcheck_polynomial would.  Power-of-two lengths >= 4 run as
 * one fused pass over the quadruples (k, k+L/4, k+L/2, k+3L/4); other lengths
 * fold then evaluate, as the reference falls back to (:194-196). */
int effsc_fused_fold_and_compute_polynomial(effsc_ctx* ctx, int field, int repr, const uint64_t* values, size_t len,
                                            int ncomp, const uint64_t* weight, uint64_t* out, size_t* out_len,
                                            uint64_t* out_s0_s1);

/* ---- eq table ----------------------------------------------------------------
 * eq(w, .) over {0,1}^num_vars in MSB layout (EqFactored's build_eq_table,
 * src/provers/eq_factored.rs:217-239), written to host `out`
 * (2^num_vars elements of `field` words). */
int effsc_build_eq_table(effsc_ctx* ctx, int field, int repr, const uint64_t* w, size_t num_vars,
                         uint64_t* out);

/* ---- seeded inputs ---------------------------------------------------------
 * The seeded uniform generator shared with the tests: element i of a table
 * with seed s is SplitMix64 output i (re-mixed while >= p), canonical.
 * Fills a device buffer (dev_out) or a host buffer (host_out). */
int effsc_gen_uniform(effsc_ctx* ctx, uint64_t seed, uint64_t n, uint64_t* dev_out, uint64_t* host_out);
uint64_t effsc_table_seed(uint64_t seed, uint64_t table);

/* Integer-pipe microbenchmark (no reference counterpart): the device's rate
 * of Goldilocks products (64x64 -> 128-bit product plus reduction) and of
 * Fp3 x Fp3 products, each from independent dependency chains in every
 * thread of a full grid; the denominator of the integer-multiply roofline. */
int effsc_diag_mulmod_rate(effsc_ctx* ctx, double* mulmod_per_s, double* fp3_mul_per_s);
/* Accumulate-form integer rates (no reference counterpart): products of
 * 64-bit operands added unreduced into independent lazy sums (two per
 * thread, the split accumulator of the folds) per second, and reductions of
 * a 160-bit sum to a canonical residue per second, each on a full grid.
 * These are the operations the round kernels execute (a product costs no
 * reduction until its sum is stored), so they bound the integer roofline:
 * products / mac_per_s + reductions / reduce_per_s. */
int effsc_diag_accumulate_rate(effsc_ctx* ctx, double* mac_per_s, double* reduce_per_s);

/* Transcript latency probe (no reference counterpart): one warp runs 1000
 * Keccak-f[1600] permutations, then 1000 round steps (send one Fp3 element,
 * squeeze one challenge); ns per permutation and per step, from the device's
 * global timer.  The per-round floor of every round of a proof. */
int effsc_diag_transcript_latency(effsc_ctx* ctx, double* ns_per_permutation, double* ns_per_round_step);

/* Self-test of the bounded wait that the TMA-staged round kernel uses on its
 * own mbarriers (no reference counterpart): one thread waits on a barrier
 * that nothing completes (arrive = 0) or that it completed itself (arrive =
 * 1), giving up after limit_ns (at most 2 s).  *status = 0 when the wait
 * completed, EFFSC_STATUS_TIMEOUT (4) when it gave up; the context stays
 * usable either way. */
int effsc_diag_bounded_wait(effsc_ctx* ctx, uint64_t limit_ns, int arrive, uint32_t* status);

/* sumcheck_verify (src/verifier.rs:61-139) for n proofs at once on the
 * device (no reference counterpart for the batch; the serving loop's
 * self-check): proof i has num_rounds[i] rounds of `degree` (0..3) wire
 * elements each, rows concatenated in proof order (round_polys: max(degree,
 * 1) elements per row, `field` canonical words per element), its claimed sum
 * and the transcript state it starts from; the same hook bytes are absorbed
 * every round.  Writes each proof's final claim (and, if challenges is not
 * NULL, the recomputed challenges per row).  The caller compares final_claim
 * with the evaluation it expects (for proofs of this library: the proof's
 * final value).  The transcripts are not modified. */
int effsc_verify_batch(effsc_ctx* ctx, int field, size_t n, const uint64_t* claimed_sums, int degree,
                       const uint32_t* num_rounds, const effsc_transcript* const* transcripts, const uint8_t* hook,
                       size_t hook_len, const uint64_t* round_polys, uint64_t* challenges, uint64_t* final_claims);

/* protogalaxy::fold (src/folding.rs:14-75): folds n_polys univariate
 * polynomials with n_levels pairs (a, b), level k replacing neighbours
 * p[2i], p[2i+1] by p[2i] + (a_k + b_k X)(p[2i+1] - p[2i]).  Release-build
 * semantics: an odd last polynomial is dropped at its level and levels after
 * a single polynomial remains change nothing (the reference debug-asserts
 * n_polys == 2^n_levels).
 *   pairs:  n_levels x (a, b), `field` canonical words per element.
 *   polys:  n_polys rows of `width` coefficients (ascending degree, zero-
 *           padded, canonical), `field` words each; device, pinned or host
 *           memory.
 *   out:    host, capacity max(width + n_levels, 1) elements; *out_len = the
 *           number of coefficients of the result with trailing zeros trimmed:
 *           0 for n_polys = 0, the input's own trimmed length for
 *           n_polys = 1, at least 1 otherwise (to_dense_poly,
 *           src/poly_ops.rs:159-166). */
int effsc_protogalaxy_fold(effsc_ctx* ctx, int field, const uint64_t* pairs, size_t n_levels, const uint64_t* polys,
                           size_t n_polys, size_t width, uint64_t* out, size_t* out_len);

/* ---- batches: many independent provers, one launch per round -------------
 * No reference counterpart (the crate proves one instance per call).  A batch
 * holds n_inst InnerProductProver (kind EFFSC_IP, tables a and b) or
 * MultilinearProver (EFFSC_ML) instances in MSB order; instance i has
 * num_vars[i] (1..34) variables and power-of-two tables of 2^num_vars[i]
 * base-field elements: host_tables[i * ntab + t] (canonical words) or, when
 * host_tables is NULL, the seeded uniform tables of effsc_gen_uniform with
 * seed seeds[i * ntab + t].  effsc_batch_prove proves every instance with all
 * num_vars[i] rounds -- runner::sumcheck (src/runner.rs:29-69) with the
 * Keccak transcript transcripts[i], no hook -- running one kernel per round
 * for all instances still active (replayed as one CUDA graph when use_graph).
 * Each proof is bit-identical to proving that instance alone.  Outputs are
 * concatenated: instance i's rounds start at row R_i = num_vars[0] + ... +
 * num_vars[i-1] (round_polys: deg elements per row, challenges: 1 element per
 * row), final_values[i]; all canonical, `field` words per element.  The
 * input tables are never written, so the batch can be proved again. */
typedef struct effsc_batch effsc_batch;
int effsc_batch_create(effsc_ctx* ctx, int kind, int field, size_t n_inst, const uint32_t* num_vars,
                       const uint64_t* const* host_tables, const uint64_t* seeds, effsc_batch** out);
int effsc_batch_destroy(effsc_batch* b);
int effsc_batch_prove(effsc_batch* b, const effsc_transcript* const* transcripts, int use_graph,
                      uint64_t* round_polys, uint64_t* challenges, uint64_t* final_values);
/* Work granularity: quadruples per thread of a round's blocks (1..64). */
int effsc_batch_set_quads_per_thread(effsc_batch* b, int quads_per_thread);
/* Tail switch: once an instance's tables are at most max_len long, its
 * remaining rounds run in one thread block (shared memory) of a single tail
 * launch for the whole batch.  Default ~0: as long as shared memory allows;
 * 0 disables. */
int effsc_batch_set_tail(effsc_batch* b, uint64_t max_len);
/* Autotuner: times quads-per-thread {1, 2, 4, 8} x tail switch {off, 2^6,
 * 2^8, 2^10, largest} on this batch, keeps the fastest and appends the
 * measurements to cache_path (JSON lines) if given. */
int effsc_batch_tune(effsc_batch* b, const effsc_transcript* const* transcripts, const char* cache_path,
                     int* quads_per_thread, uint64_t* tail_len);
/* Device address of instance inst's input table (2^num_vars canonical words). */
int effsc_batch_device_table(effsc_batch* b, size_t inst, int table, const uint64_t** out);

/* ---- serving: a request loop with continuous batching ---------------------
 * No reference counterpart.  Requests (MSB InnerProduct or Multilinear
 * proofs, all num_vars rounds, the Keccak transcript `t` as it stands at
 * submission, no hook) queue FIFO.  effsc_server_progress admits queued
 * requests while fewer than max_active are in flight and their device memory
 * (tables, Fp3 work buffers, proof and transcript state) fits in
 * hbm_budget_bytes, then launches one step: a single kernel in which every
 * admitted request advances one round or finalises.  Finished proofs are
 * returned by effsc_server_take in completion order.  Each proof is
 * bit-identical to proving the request alone (runner::sumcheck,
 * src/runner.rs:29-69).  Host tables (host_tables[k], 2^num_vars canonical
 * words) must stay valid until the request is admitted; with host_tables NULL
 * the tables are generated on the device from seeds[k] (effsc_gen_uniform).
 * Not thread-safe: one host thread drives a server. */
typedef struct effsc_server effsc_server;
int effsc_server_create(effsc_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t max_active, effsc_server** out);
int effsc_server_destroy(effsc_server* s);
int effsc_server_submit(effsc_server* s, int kind, int field, uint32_t num_vars, const uint64_t* const* host_tables,
                        const uint64_t* seeds, const effsc_transcript* t, uint64_t* id);
/* Admit, launch one step, collect finished proofs.  wait != 0: block until at
 * least one proof is finished if any is in flight.  *pending: requests not
 * yet taken (queued, active or finishing). */
int effsc_server_progress(effsc_server* s, int wait, uint32_t* pending);
/* Oldest finished proof: *id (~0 when none), num_vars rows of round_polys
 * (degree x field words) and challenges (field words), final_value (field
 * words); seconds queued and seconds from submission to completion. */
int effsc_server_take(effsc_server* s, uint64_t* id, uint32_t* num_vars, uint64_t* round_polys, uint64_t* challenges,
                      uint64_t* final_value, double* queue_s, double* latency_s);
/* Open-loop driver: request i (kinds[i], num_vars[i], seeds[2i..2i+1],
 * transcripts[i]) is submitted arrival_s[i] seconds after the start; runs
 * until every proof is finished.  latency_s[i] = completion - arrival; the
 * proofs are concatenated in request order: request i's rounds start at row
 * R_i = num_vars[0] + ... + num_vars[i-1], a round_polys row holds 2
 * elements (Multilinear rows: [h(0), 0]), a challenges row 1 element; NULL
 * outputs are skipped. */
int effsc_server_run_trace(effsc_server* s, size_t n, const int* kinds, int field, const uint32_t* num_vars,
                           const uint64_t* seeds, const effsc_transcript* const* transcripts, const double* arrival_s,
                           double* latency_s, double* makespan_s, uint64_t* round_polys, uint64_t* challenges,
                           uint64_t* final_values);
/* The same driver with every request's tables in host memory (the serving
 * case where inputs arrive over the host link): request i's tables are
 * host_tables[2i] and, for an InnerProduct request, host_tables[2i + 1]
 * (2^num_vars[i] canonical words each; pinned memory uploads fastest), and
 * the upload joins the request's latency. */
int effsc_server_run_trace_host(effsc_server* s, size_t n, const int* kinds, int field, const uint32_t* num_vars,
                                const uint64_t* const* host_tables, const effsc_transcript* const* transcripts,
                                const double* arrival_s, double* latency_s, double* makespan_s, uint64_t* round_polys,
                                uint64_t* challenges, uint64_t* final_values);

/* ---- one round without allocation -----------------------------------------
 * No counterpart in the reference.  For callers that must not allocate device
 * memory (a host application whose own pool has reserved the HBM, or work
 * sharing a stream with latency-critical kernels that a synchronising
 * cudaMalloc/cudaFree would stall): one InnerProductProver (MSB) round on the
 * caller's device buffers -- challenge == NULL evaluates round 0 on a, b
 * (len >= 1); otherwise folds a, b with *challenge and evaluates the next
 * round (len a power of two >= 4).  challenge points to 3 words in HOST
 * memory (one Fp3 element, read before the call returns; words >= p are
 * reduced mod p).  a, b: Fp3 tables of len
 * elements in structure-of-arrays form (c0[len], c1[len], c2[len], canonical);
 * the folded tables go to the first len/2 entries of each component array of
 * a_out, b_out (same component stride len; a_out == a works in place).
 * out_evals: 6 device words [q(0), q(inf)], valid once the stream has run the
 * call.  The grid reduction uses a static device array sized for at most 4096
 * blocks (about 384 KiB, held by every GPU that loads the library); blocks = 0
 * picks the grid, blocks > 4096 is rejected.  The first call on a device
 * resolves that array's address, so make it before any stream capture.  All
 * calls share the array: calls that overlap on the GPU (other streams,
 * threads) race and must be serialised by the caller.  Issues no cudaMalloc
 * or cudaFree and does not synchronise. */
int effsc_ip_round_noalloc(const uint64_t* a, const uint64_t* b, uint64_t* a_out, uint64_t* b_out,
                           size_t len, const uint64_t* challenge, uint64_t* out_evals, int blocks, void* stream);

/* ---- device memory helpers (for the device-resident constructors) ------- */
int effsc_device_alloc(effsc_ctx* ctx, size_t bytes, void** out);
int effsc_device_free(effsc_ctx* ctx, void* ptr);
int effsc_memcpy_h2d(effsc_ctx* ctx, void* dst, const void* src, size_t bytes);
int effsc_memcpy_d2h(effsc_ctx* ctx, void* dst, const void* src, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
