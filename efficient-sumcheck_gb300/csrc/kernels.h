// kernels.h -- launch interface between the host runtime and the sumcheck
// round kernels.  Internal to the library (not part of the C ABI).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

typedef unsigned long long u64;
typedef unsigned int u32;

namespace effsc {

// Threads per block of every round kernel.
constexpr int KERNEL_TPB = 256;

// Kernels of a proof's chain are launched with programmatic dependent launch:
// a kernel may be scheduled while the previous kernel on the stream drains
// (its last block's reduction and transcript step), and waits on the device
// (griddepcontrol.wait, the first statement of every such kernel) before it
// touches memory.  EFFSC_PDL=0 in the environment launches them plainly.
bool pdl_on(void);
template <class... KArgs, class... Args>
inline bool launch_chain(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                         Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_on() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...) == cudaSuccess;
}
int max_grid(void);
// One wave of a grid-stride kernel: the blocks the SMs hold at once (the
// occupancy calculator's count for KERNEL_TPB threads and `smem` bytes per
// block, cached per kernel and device, times the SM count).  The streaming
// round kernels measured faster as one wave than as several (InnerProduct's
// second pass, the Coefficient eq * f * g rounds).
template <auto Kernel>
inline int one_wave(size_t smem) {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return max_grid();
    int& c = cached[dev & 63];
    if (c > 0) return c;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, Kernel, KERNEL_TPB, smem) != cudaSuccess || nb < 1) {
        cudaGetLastError();
        return max_grid();
    }
    c = nb * (max_grid() / 8);
    return c;
}
// A grid of at most one wave of Kernel.
template <auto Kernel>
inline int wave_grid(int grid, size_t smem = 0) {
    const int w = one_wave<Kernel>(smem);
    return grid < w ? grid : w;
}
// Value a kernel writes to RoundArgs::status when a bounded wait times out.
constexpr unsigned EFFSC_STATUS_TIMEOUT = 4;

// Fold / evaluate semantics.
//  SEM_MSB_PAD  : half = next_pow2(L)/2, unpaired tail folds as v*(1-w)
//                 (reference src/inner_product_sumcheck.rs:143-176)
//  SEM_MSB_FLOOR: half = L/2, no tail (src/provers/coefficient.rs:131-140)
//  SEM_LSB      : pairs (2k, 2k+1), floor(L/2) outputs
//                 (src/provers/multilinear_lsb.rs:141-166)
enum Sem { SEM_MSB_PAD = 0, SEM_MSB_FLOOR = 1, SEM_LSB = 2 };

// Round-polynomial policies (what is accumulated per pair).
//  POL_ML  : s0 = sum lo, s1 = sum hi                       (1 table)
//  POL_IP  : q0 = sum lo_a lo_b, qinf = sum (da)(db)        (2 tables)
//  POL_C1..3: coefficients of prod_i (lo_i + x d_i)         (1..3 tables)
//  POL_EQFR: POL_IP on (eq_r, p), times the scalar eq_l[0]  (2 tables)
//  POL_IP01: InnerProduct rounds 0 and 1 from one pass over the base tables
//            (eight base-field sums, two transcript steps)
//  POL_C3W : POL_C3 without h(1) (the wire needs h(0), h(inf), h(2); the
//            legacy (c0, c1) pair is not produced): the device protocol
//  POL_ML01: Multilinear rounds 0 and 1 from one pass (quarter sums)
//  POL_GKR : GkrProver, q(0) and the x^2 coefficient of the quadratic
//            add (W_b + W_c) + mult W_b W_c: the wire [q(0), q(inf)]
enum Pol {
    POL_ML = 0, POL_IP = 1, POL_C1 = 2, POL_C2 = 3, POL_C3 = 4, POL_EQFR = 5, POL_EQFL = 6, POL_IP01 = 7,
    POL_GKR = 8, POL_C3W = 9, POL_ML01 = 10,
    // CoefficientProver with a declarative evaluator (ExprProgram) of degree
    // 1, 2, 3: raw values are the coefficients c0..c3
    POL_X1 = 11, POL_X2 = 12, POL_X3 = 13
};

// A declarative RoundPolyEvaluator (src/coefficient_sumcheck.rs:50-76): per
// pair, coeffs[coeff] += k * prod of the factors, each factor the even (lo)
// or odd (hi) element of a column.  Columns are the pairwise tables and the
// columns of the tablewise tables (a tablewise row is one element of each of
// its columns).  factor = column * 2 + (0: even, 1: odd).
constexpr int EXPR_MAX_TERMS = 16;
constexpr int EXPR_MAX_FACTORS = 4;
struct ExprTerm {
    unsigned char coeff, nf;
    unsigned char f[EXPR_MAX_FACTORS];
    u64 k[3];               // canonical Fp3 constant
};
struct ExprProgram {
    u32 nterms, degree, ncols;
    ExprTerm t[EXPR_MAX_TERMS];
};

struct TabIO {
    const u64* in[3];   // SoA component arrays; [1],[2] null for base tables
    u64* out[3];
};

// Optional transcript step performed by the last block of a round kernel.
struct TxIO {
    void* tx;              // DevTranscript* (null: no transcript step)
    const uint8_t* hook;   // bytes absorbed after the round's messages
    u32 hook_len;
    u64* proof_wire;       // where the round's wire values go (d * 3 words)
    u64* proof_chal;       // where the squeezed challenge goes (3 words)
    u64* chal_next;        // challenge slot read by the next round (3 words)
};

struct RoundArgs {
    TabIO t[4];
    u64 L;                 // length before folding (fold/fused) or current length (eval)
    u32 m_shift;           // EqFactored left phase: log2 |eq_r|; GkrProver: k = log2 |W|
    u64 el_len;            // EqFactored left phase: current |eq_l|
    const u64* chal_ptr;   // challenge in device memory, or null to use `chal`
    const u64* chal2_ptr;  // second challenge (InnerProduct double fold of round 2)
    u64 chal[3];
    const u64* scalar[3];  // EqFactored right phase: eq_l[0] (c1, c2 null if base)
    u64* partials;         // gridDim * 12 words
    u32* counter;          // zero between launches (the last block resets it)
    u64* result;           // wire (d*3 words) then aux pair (6 words)
    u32* status;           // device status word (non-zero: error code)
    TxIO tx;
    // the first pass of the InnerProduct start over a chunk of the tables:
    // its tiles start at tile0, and its 26 sums go to `acc` (ACC_FIRST),
    // are added there (ACC_MID) or are added and finalised (ACC_LAST)
    u32 tile0;
    u32 acc_mode;
    u64* acc;
};
enum AccMode { ACC_NONE = 0, ACC_FIRST = 1, ACC_MID = 2, ACC_LAST = 3 };


// The last rounds of an MSB Multilinear / InnerProduct proof run by one block
// with the tables in shared memory: rounds r0 .. r0 + nrounds - 1, each a
// fold with the previous challenge (except a first round 0) plus evaluation,
// block reduction and the transcript step, without a kernel boundary.
struct TailArgs {
    const u64* in[3][3];   // [table][component] current tables (length L)
    u64* out[3][3];        // tables after the tail's last fold (null: none)
    u64 L;                 // power of two, length at the start of round r0
    u32 in_ext;            // bit t: table t is stored with 3 components
    u32 nrounds;
    u32 first_fold;        // 1: the first round folds with chal_in first
    u32 hook_len;
    const u64* chal_in;    // challenge of the round before r0 (3 words)
    void* tx;              // DevTranscript*
    const uint8_t* hook;
    u64* proof_wire;       // round r0's wire values (3 * nwire words per round)
    u64* proof_chal;       // round r0's challenge (3 words per round)
    u32 final_fold;        // 1: the runner's finalize (one more fold with the last
                           // challenge) before the tables are written back
    u64* first_out;        // (optional) the tables' first entries, 3 words per table, 4 tables
    u32 lsb;               // LSB prover: pairs (2j, 2j+1); held bit-reversed in shared memory
};
// Largest table length (a power of two) the tail kernel holds for this
// policy and field width (1: Fp, 3: Fp3), within `smem_cap` bytes.
u64 tail_max_len(int pol, int fw, u64 smem_cap);
constexpr u64 TAIL_SMEM_CAP = 200 * 1024;
// One block per TailArgs; `smem_len` = largest L among them.
bool launch_tail(int pol, int fw, const TailArgs* dev_args, const TailArgs* one, u32 n, u64 smem_len, cudaStream_t s);
// Cluster tail: 2^cs_log CTAs hold a table of a.L entries (a.L >> cs_log per
// CTA within TAIL_SMEM_CAP); needs a.first_fold = 1 and a.nrounds > cs_log + 1.
bool launch_tail_cluster(int pol, int fw, const TailArgs& a, u32 cs_log, cudaStream_t s);
// Largest cluster size the device runs for it (16, 8 or 0).
u32 tail_cluster_max(void);

// GkrProver tail (k_gkr_tail.cu): add, mult, W_b, W_c in one block's shared
// memory for the rounds r0 .. r0 + nrounds - 1, then the runner's finalize.
struct GkrTailArgs {
    const u64* in[4][3];   // [table][component] current add, mult, W_b, W_c
    u64* out[4][3];        // the tables after the last fold (null: not written)
    u64 len[4];            // current lengths (powers of two)
    u32 in_ext;            // bit t: table t is stored with 3 components
    u32 nrounds;
    u32 r0;                // index of the first tail round (W_b folds while the bound variable is < k)
    u32 k;                 // log2 |w|
    u32 first_fold;        // 1: the first round folds with chal_in first
    u32 final_fold;        // 1: the runner's finalize before the tables are written back
    u32 hook_len;
    const u64* chal_in;
    void* tx;              // DevTranscript*
    const uint8_t* hook;
    u64* proof_wire;       // round r0's wire values (6 words per round)
    u64* proof_chal;       // round r0's challenge (3 words per round)
    u64* first_out;        // (optional) the four tables' first entries, 3 words each
};
// Needs 8 * fw * (len[0] + .. + len[3]) bytes <= TAIL_SMEM_CAP.
bool launch_gkr_tail(int fw, const GkrTailArgs& a, u64 smem_bytes, cudaStream_t s);

// Serving steps: one entry per request in the step, sorted by first_block;
// `code` = SERVE_IP (else ML) | SERVE_FP3 (else Fp) | phase << SERVE_PHASE_SHIFT.
struct ServeSeg {
    u32 first_block;
    u32 nblocks;
    u32 code;
    u32 reserved;
};
constexpr u32 SERVE_IP = 1, SERVE_FP3 = 2, SERVE_PHASE_SHIFT = 2;
// SERVE_IP01 / SERVE_IP2X: InnerProduct rounds 0-1 / round 2 of the two-pass
// start (Fp3 challenges, base tables; ip01.cuh).
enum ServePhase {
    SERVE_EVAL = 0, SERVE_FOLD_BASE = 1, SERVE_FOLD_EXT = 2, SERVE_FINAL_BASE = 3, SERVE_FINAL_EXT = 4,
    SERVE_IP01 = 5, SERVE_IP2X = 6
};
void launch_serve_step(const ServeSeg* segs, u32 nsegs, const RoundArgs* args, u32 grid, cudaStream_t s);

// EqFactored left phase from the inner sums (k_eqf.cu).  A Tab3 holds a
// table's component arrays (components 1, 2 unused for base tables).
struct Tab3 {
    const u64* c[3];
};
void launch_eqf_inner(bool ee, bool ep, Tab3 p, Tab3 er, u64 m, u64 rows, u64* s0, u64* s1, u64* s2, cudaStream_t s);
// out = p folded over its top log2(rows) variables with the eq weights e
// (rows x Lc entries of p; splits row groups summed through `part`, 3 words
// per entry per split).
void launch_eqf_fold_rows(bool ew, bool ep, Tab3 p, Tab3 e, u64 Lc, u64 rows, u64 splits, u64* part, int fw, u64* o0,
                          u64* o1, u64* o2, cudaStream_t s);

int pol_ntables(int pol);
int pol_nraw(int pol);
int pol_nwire(int pol);

// Returns false if no kernel is instantiated for this combination.
bool launch_fold(int sem, bool ein, bool ech, const RoundArgs& a, int t, int grid, cudaStream_t s);
// Round polynomial of a declarative evaluator on the current columns
// (a.t[0..ncols), a.L entries each; MSB floor pairs (k, k + L/2) or LSB pairs
// (2k, 2k+1)); the last block finalises with policy POL_X<degree>.
bool launch_expr_eval(int sem, const RoundArgs& a, const ExprProgram& prog, int grid, cudaStream_t s);
bool launch_eval(int pol, int sem, u32 mask, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_fused(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_eqf_left(bool fused, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s);
// TMA-staged fused MSB round: tiles of KERNEL_TPB quadruples; returns false
// if no kernel is instantiated for the combination.
bool launch_fused_tma(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, u32 ntiles, int grid, cudaStream_t s);
int fused_tma_blocks_per_sm(void);
// GkrProver round: t[0] = add, t[1] = mult (both Fp3 when ea), t[2] = W_b,
// t[3] = W_c (Fp3 when ew; the compact witness tables of 2^(k - bound b
// variables) and 2^(k - bound c variables) entries).  fused: fold add and
// mult with the challenge (L a power of two >= 4) and evaluate the folded
// tables; otherwise evaluate the current ones.
bool launch_gkr(bool fused, bool ea, bool ewb, bool ewc, bool ech, const RoundArgs& a, int grid, cudaStream_t s);
// InnerProduct (MSB or LSB) over Fp3 challenges, base tables of length L = 2^n >= 8:
// rounds 0 and 1 from one read of the tables (launch_ip01), then round 2's
// fold-twice-and-evaluate from a second read (launch_ip2x).
bool launch_ip01(bool lsb, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_ip2x(bool lsb, const RoundArgs& a, int grid, cudaStream_t s);
// InnerProduct rounds 0-3 in two passes (k_ip012.cu): rounds 0, 1 and 2 from
// 26 base-field sums of one read of the tables (launch_ip012; partials of 32
// words per block, grid at most max_grid() * 3 / 8 blocks), then the fold with r0,
// r1, r2 at once and round 3 from a second read (launch_ip3x; a.chal_ptr
// holds r0, r1, r2 as 9 consecutive words).
bool launch_ip012(bool lsb, const RoundArgs& a, int grid, cudaStream_t s);
// The first pass over tables in host memory that also copies them to the
// device buffers a.t[0].out[0], a.t[1].out[0] (L words each, 16-byte aligned)
// for the second pass.
bool launch_ip012_mirror(bool lsb, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_ip3x(bool lsb, const RoundArgs& a, int grid, cudaStream_t s);
// The first pass with the tables streamed through shared memory by bulk
// copies: ntiles = (L/8) / ip012_tile_octets() tiles; device-memory tables,
// 16-byte aligned; at most two blocks per SM for the partials.  (The second
// pass keeps direct loads: staged, it measured slower.)
bool launch_ip012_staged(bool lsb, const RoundArgs& a, u32 ntiles, int grid, cudaStream_t s);
u32 ip012_tile_octets(void);
// Consecutive InnerProduct rounds over Fp3 tables in one cooperative launch
// (k_persist.cu): round k of the launch folds tables of length L0 >> k with
// the previous challenge and evaluates; the last block to reach the grid
// barrier runs the transcript step.  a.tx carries the transcript and hook,
// a.partials (grid * RAW_WORDS words) and a.status as for the other round
// kernels.
struct PersistArgs {
    u32 nrounds;          // rounds run by this launch
    u64 L0;               // table length before the first round's fold
    const u64* chal_in;   // the challenge before the first round (3 words)
    u64* proof_wire;      // the first round's wire row (6 words per round)
    u64* proof_chal;      // the first round's challenge (3 words per round)
    u32* bar;             // barrier: [0] arrivals (zero between launches), [1] generation
    u64* buf[2][2][3];    // [ping-pong][table][component]: MSB folds [0] in place
};
bool launch_ip_persist(bool lsb, const RoundArgs& a, const PersistArgs& p, int grid, cudaStream_t s);
int persist_max_grid(bool lsb);
// Coefficient rounds 0-2 in two passes (k_coef01.cu; degree-3 product
// evaluator over three tables, table 0 in Fp (e0 false) or Fp3, tables 1-2 in
// Fp, Fp3 challenges): rounds 0 and 1 from 15 sums of one read (partials of
// 48 words per block, so at most max_grid() / 4 blocks), then the fold with
// r0 and r1 at once (a.chal_ptr, a.chal2_ptr) and round 2 from a second read.
bool launch_c3_r01(bool lsb, bool e0, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_c3_r2x(bool lsb, bool e0, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_ml01(const RoundArgs& a, int grid, cudaStream_t s);
bool launch_ml2x(bool ech, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_gkr01(const RoundArgs& a, int grid, cudaStream_t s);
// The same pass by runs at three blocks per SM: only when each lane gets a run of at least
// two quadruples inside one W_b entry (grid * TPB / 32 warps, |w| >= 64 * 2).
bool launch_gkr01_runs(const RoundArgs& a, int grid, cudaStream_t s);
bool launch_gkr2x(bool ech, const RoundArgs& a, int grid, cudaStream_t s);
void launch_batch_finalize(const RoundArgs* args, const unsigned char* ext, u32 n, int ntab, u64* finals, cudaStream_t s);

// Utility kernels.
void launch_split_aos(const u64* aos, u64 n, int ncomp, u64* c0, u64* c1, u64* c2, int from_mont, u32* ext_flag, cudaStream_t s);
void launch_join_aos(const u64* c0, const u64* c1, const u64* c2, u64 n, int ncomp, u64* aos, int to_mont, cudaStream_t s);
void launch_copy(const u64* src, u64* dst, u64 n, cudaStream_t s);
// dst[3 t + c] = p[t][c][0] for the non-null component pointers, else 0.
struct FirstSrc {
    const u64* p[4][3];
};
void launch_gather_first(const FirstSrc& src, u64* dst, cudaStream_t s);
void launch_fill(u64* dst, u64 n, u64 v, cudaStream_t s);
bool launch_build_eq(const u64* w, u32 v, int ext, u64* c0, u64* c1, u64* c2, cudaStream_t s);
void launch_gen_uniform(u64 seed, u64 n, u64* out, cudaStream_t s);
bool diag_mulmod_rate(cudaStream_t s, double* mulmod_per_s, double* fp3_mul_per_s);
bool diag_accumulate_rate(cudaStream_t s, double* mac_per_s, double* reduce_per_s);
// One thread waits on an mbarrier with the round kernels' bounded wait;
// `arrive`: complete the phase first.  *status = 0 or EFFSC_STATUS_TIMEOUT.
void launch_diag_bounded_wait(u64 limit_ns, int arrive, u32* status, cudaStream_t s);
void launch_diag_transcript(u32 iters, u64* out, cudaStream_t s);
int max_grid(void);
void kernels_init(int device);

}  // namespace effsc

// Sets the thread-local message returned by effsc_last_error(); returns code.
int effsc_set_error(int code, const char* fmt, ...);

namespace effsc {

}  // namespace effsc
