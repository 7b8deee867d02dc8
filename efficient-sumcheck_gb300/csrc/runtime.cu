// runtime.cu -- host runtime behind the C ABI (include/effsc_gpu.h).
//
// Owns device tables, dispatches each prover round to the kernels of
// k_mlip.cu / k_coef.cu / k_misc.cu, runs the whole protocol on the device
// (optionally as a CUDA graph), and implements the host transcript and the
// verifier.  Each prover's round logic restates the reference prover it
// replaces (file:line cited at each branch).
#include "effsc_gpu.h"
#include "kernels.h"
#include "keccak.cuh"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <map>
#include <mutex>

using namespace effsc;

// ===========================================================================
// errors
// ===========================================================================
namespace {
thread_local std::string g_err;
thread_local uint64_t g_launches = 0;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
}  // namespace

int effsc_set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(EFFSC_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
#define TRY(call)                   \
    do {                            \
        int r_ = (call);            \
        if (r_ != EFFSC_OK) return r_; \
    } while (0)

// ===========================================================================
// host field arithmetic (boundary conversions, final values, verifier)
// ===========================================================================
namespace {
typedef unsigned __int128 u128;
const u64 HP = 0xFFFFFFFF00000001ULL;
const u64 HEPS = 0xFFFFFFFFULL;
const u64 HW = 0xFFFFFFF800000001ULL;
const u64 HR_INV = 0xFFFFFFFF00000001ULL - (1ULL << 32);

inline u64 h_reduce128(u128 x) {
    u64 lo = (u64)x, hi = (u64)(x >> 64);
    u64 hh = hi >> 32, hl = hi & HEPS;
    u64 t0 = lo - hh;
    if (lo < hh) t0 -= HEPS;
    u64 t1 = hl * HEPS;
    u64 t2 = t0 + t1;
    if (t2 < t1) t2 += HEPS;
    return t2 >= HP ? t2 - HP : t2;
}
inline u64 h_add(u64 a, u64 b) { u64 s = a + b; if (s < a) return s + HEPS; return s >= HP ? s - HP : s; }
inline u64 h_sub(u64 a, u64 b) { u64 d = a - b; return a < b ? d - HEPS : d; }
inline u64 h_mul(u64 a, u64 b) { return h_reduce128((u128)a * b); }
u64 h_pow(u64 a, u64 e) { u64 r = 1; while (e) { if (e & 1) r = h_mul(r, a); a = h_mul(a, a); e >>= 1; } return r; }
inline u64 h_inv(u64 a) { return h_pow(a, HP - 2); }

struct HF { u64 c[3]; };
inline HF hf(u64 a, u64 b = 0, u64 c = 0) { HF r; r.c[0] = a; r.c[1] = b; r.c[2] = c; return r; }
inline HF hf_add(HF a, HF b) { return hf(h_add(a.c[0], b.c[0]), h_add(a.c[1], b.c[1]), h_add(a.c[2], b.c[2])); }
inline HF hf_sub(HF a, HF b) { return hf(h_sub(a.c[0], b.c[0]), h_sub(a.c[1], b.c[1]), h_sub(a.c[2], b.c[2])); }
inline HF hf_mul(HF a, HF b) {
    u64 a0 = a.c[0], a1 = a.c[1], a2 = a.c[2], b0 = b.c[0], b1 = b.c[1], b2 = b.c[2];
    return hf(h_add(h_mul(a0, b0), h_mul(HW, h_add(h_mul(a1, b2), h_mul(a2, b1)))),
              h_add(h_add(h_mul(a0, b1), h_mul(a1, b0)), h_mul(HW, h_mul(a2, b2))),
              h_add(h_add(h_mul(a0, b2), h_mul(a1, b1)), h_mul(a2, b0)));
}
inline HF hf_from_u64(u64 x) { return hf(x % HP); }
inline bool hf_is_ext(const HF& a) { return (a.c[1] | a.c[2]) != 0; }

inline u64 to_canon(u64 x, int repr) { x = x >= HP ? x - HP : x; return repr == EFFSC_MONTGOMERY ? h_mul(x, HR_INV) : x; }
inline u64 from_canon(u64 x, int repr) { return repr == EFFSC_MONTGOMERY ? h_mul(x, HEPS) : x; }
// Read one element of `field` words in `repr` into canonical Fp3.
inline HF load_elem(const uint64_t* p, int field, int repr) {
    HF r = hf(to_canon(p[0], repr));
    if (field == EFFSC_FP3) { r.c[1] = to_canon(p[1], repr); r.c[2] = to_canon(p[2], repr); }
    return r;
}
inline void store_elem(uint64_t* p, const HF& v, int field, int repr) {
    p[0] = from_canon(v.c[0], repr);
    if (field == EFFSC_FP3) { p[1] = from_canon(v.c[1], repr); p[2] = from_canon(v.c[2], repr); }
}

// ===========================================================================
// host Keccak-f[1600] and the duplex transcript (same construction as
// keccak.cuh; FIPS 202 permutation)
// ===========================================================================
const u64 K_RC[24] = {
    0x0000000000000001ULL, 0x0000000000008082ULL, 0x800000000000808AULL, 0x8000000080008000ULL,
    0x000000000000808BULL, 0x0000000080000001ULL, 0x8000000080008081ULL, 0x8000000000008009ULL,
    0x000000000000008AULL, 0x0000000000000088ULL, 0x0000000080008009ULL, 0x000000008000000AULL,
    0x000000008000808BULL, 0x800000000000008BULL, 0x8000000000008089ULL, 0x8000000000008003ULL,
    0x8000000000008002ULL, 0x8000000000000080ULL, 0x000000000000800AULL, 0x800000008000000AULL,
    0x8000000080008081ULL, 0x8000000000008080ULL, 0x0000000080000001ULL, 0x8000000080008008ULL};
const int K_ROT[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43, 25, 39, 41, 45, 15, 21, 8, 18, 2, 61, 56, 14};
inline u64 rotl(u64 x, int r) { return r ? (x << r) | (x >> (64 - r)) : x; }
void keccak_f(u64* A) {
    for (int round = 0; round < 24; round++) {
        u64 C[5], B[25];
        for (int x = 0; x < 5; x++) C[x] = A[x] ^ A[x + 5] ^ A[x + 10] ^ A[x + 15] ^ A[x + 20];
        for (int x = 0; x < 5; x++) {
            u64 D = C[(x + 4) % 5] ^ rotl(C[(x + 1) % 5], 1);
            for (int y = 0; y < 5; y++) A[x + 5 * y] ^= D;
        }
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) B[y + 5 * ((2 * x + 3 * y) % 5)] = rotl(A[x + 5 * y], K_ROT[x + 5 * y]);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) A[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
        A[0] ^= K_RC[round];
    }
}
}  // namespace

struct effsc_transcript {
    int kind, field, repr;
    DevTranscript st;
    u64 sm;
};

namespace {
void tx_h_absorb(effsc_transcript* t, const uint8_t* d, size_t n) {
    if (t->kind != EFFSC_T_KECCAK) return;
    DevTranscript& s = t->st;
    if (s.squeezing) { s.pos = 0; s.squeezing = 0; }
    for (size_t i = 0; i < n; i++) {
        if (s.pos == TX_RATE) { keccak_f(s.st); s.pos = 0; }
        s.st[s.pos >> 3] ^= (u64)d[i] << (8 * (s.pos & 7));
        s.pos++;
    }
}
void tx_h_squeeze(effsc_transcript* t, uint8_t* out, size_t n) {
    DevTranscript& s = t->st;
    if (!s.squeezing) {
        if (s.pos == TX_RATE) { keccak_f(s.st); s.pos = 0; }
        s.st[s.pos >> 3] ^= (u64)0x06 << (8 * (s.pos & 7));
        s.st[(TX_RATE - 1) >> 3] ^= (u64)0x80 << (8 * ((TX_RATE - 1) & 7));
        keccak_f(s.st);
        s.pos = 0;
        s.squeezing = 1;
    }
    for (size_t i = 0; i < n; i++) {
        if (s.pos == TX_RATE) { keccak_f(s.st); s.pos = 0; }
        out[i] = (uint8_t)(s.st[s.pos >> 3] >> (8 * (s.pos & 7)));
        s.pos++;
    }
}
void tx_h_send(effsc_transcript* t, const HF& v) {
    if (t->kind != EFFSC_T_KECCAK) return;
    uint8_t b[24];
    int n = t->field;
    for (int c = 0; c < n; c++)
        for (int i = 0; i < 8; i++) b[8 * c + i] = (uint8_t)(v.c[c] >> (8 * i));
    tx_h_absorb(t, b, 8 * (size_t)n);
}
HF tx_h_challenge(effsc_transcript* t) {
    if (t->kind == EFFSC_T_TEST) {
        t->sm += 0x9E3779B97F4A7C15ULL;
        u64 z = t->sm;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return hf_from_u64(z);
    }
    HF r = hf(0);
    for (int c = 0; c < t->field; c++) {
        uint8_t b[16];
        tx_h_squeeze(t, b, 16);
        u64 lo = 0, hi = 0;
        for (int i = 0; i < 8; i++) { lo |= (u64)b[i] << (8 * i); hi |= (u64)b[8 + i] << (8 * i); }
        r.c[c] = h_reduce128(((u128)hi << 64) | lo);
    }
    return r;
}
}  // namespace

// ===========================================================================
// context
// ===========================================================================
struct effsc_ctx {
    int device;
    cudaStream_t stream;
    cudaStream_t own;
    // pinned, mapped host blocks returned by destroyed provers, by size, for
    // the next provers (pinned allocation costs far more than a proof's
    // small outputs)
    std::mutex pin_mu;
    std::multimap<size_t, void*> pin_free;
};

namespace {
void* pinned_get(effsc_ctx* c, size_t bytes) {
    {
        std::lock_guard<std::mutex> g(c->pin_mu);
        auto it = c->pin_free.find(bytes);
        if (it != c->pin_free.end()) {
            void* p = it->second;
            c->pin_free.erase(it);
            return p;
        }
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocMapped) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return p;
}
void pinned_put(effsc_ctx* c, void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> g(c->pin_mu);
    if (c->pin_free.size() < 64) c->pin_free.emplace(bytes, p);
    else cudaFreeHost(p);
}
}  // namespace

// ===========================================================================
// prover state
// ===========================================================================
namespace {
struct Buf {
    u64* p[3] = {nullptr, nullptr, nullptr};
    size_t cap = 0;
    bool ext = false;
    bool owned = true;
    bool host = false;      // the caller's host memory, read in place (never bulk-copied)
};
struct Table {
    std::vector<Buf> bufs;  // bufs[0]: the input table, never written by a round
    int cur = 0;
    size_t len = 0;
    bool ext = false;
};
struct TabState {
    int cur;
    size_t len;
    bool ext;
};
}  // namespace

constexpr int UPLOAD_CHUNKS = 16;

struct effsc_prover {
    effsc_ctx* ctx = nullptr;
    int kind = 0, order = 0, field = 1, repr = 0;
    int ntab = 0;
    Table t[4];                                // GkrProver: add, mult, W_b, W_c
    size_t v = 0, v_l = 0, rounds = 0;        // EqFactored: t[0] = p, t[1] = eq_l, t[2] = eq_r
                                               // GkrProver: v = 2k, v_l = k
    size_t len0[4] = {0, 0, 0, 0};
    bool ext0[4] = {false, false, false, false};
    u64* partials = nullptr;
    // effsc_prove: InnerProduct Fp3 rounds whose tables hold at most this
    // many entries run in one cooperative launch (0: never); its grid barrier
    u64 persist_len = 0;
    u32* d_bar = nullptr;
    // host tables: copy to the device during the first pass (-1 undecided)
    int mirror = -1;
    // pinned host tables: uploaded in chunks on a copy stream while the first
    // pass runs over the chunks already on the device
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t chunk_ev[UPLOAD_CHUNKS + 1] = {};
    u64* d_acc = nullptr;
    u32* counter = nullptr;
    u32* status = nullptr;
    u64* h_res = nullptr;                      // mapped pinned: wire (9 words) + aux (6 words)
    u64* d_res = nullptr;
    DevTranscript* d_tx = nullptr;
    uint8_t* d_hook = nullptr;
    size_t hook_cap = 0;
    u64* d_wire = nullptr;
    u64* d_chals = nullptr;
    size_t rounds_cap = 0;
    // CUDA graph of a whole proof started from the reset state
    cudaGraphExec_t gexec = nullptr;
    size_t g_rounds = 0, g_hook = 0;
    uint64_t g_kernels = 0;                    // kernel nodes in the graph
    TabState g_post[4];
    size_t g_post_rounds = 0;
    // effsc_prove: tables of at most this length finish in the one-block tail
    // kernel (SIZE_MAX: as large as shared memory allows; 0: never)
    size_t tail_len = SIZE_MAX;
    // effsc_prove: 0 = one pass per round; 1 = InnerProduct rounds 0-2 in
    // two passes (k_ip01.cu), the Multilinear and GkrProver starts, the
    // EqFactored left phase from the inner sums (k_eqf.cu); 2 = as 1, with
    // InnerProduct rounds 0-3 in two passes (k_ip012.cu) where they apply
    int fuse_first = 2;
    // CoefficientProver with a declarative evaluator: the term program over
    // the columns (pairwise tables, then the tablewise tables' columns);
    // bit c of tw_cols: column c belongs to a tablewise table
    bool expr = false;
    ExprProgram prog;
    u32 tw_cols = 0;
    int n_pairwise = 0;
    u64* eqf_scratch = nullptr;               // inner sums, eq weights, partial sums
    size_t eqf_cap = 0;
    // effsc_prove outputs: pinned staging (wire | challenges | transcript |
    // first entries of the tables) and the device copy of the first entries
    u64* h_out = nullptr;
    size_t h_out_bytes = 0;
    u64* d_first = nullptr;
};

namespace {

int degree_of(const effsc_prover* p) {
    switch (p->kind) {
    case EFFSC_ML: return 1;
    case EFFSC_COEF: return p->expr ? (int)p->prog.degree : p->ntab;
    default: return 2;
    }
}
int pol_of(const effsc_prover* p) {
    switch (p->kind) {
    case EFFSC_ML: return POL_ML;
    case EFFSC_IP: return POL_IP;
    case EFFSC_COEF: return p->ntab == 1 ? POL_C1 : p->ntab == 2 ? POL_C2 : POL_C3;
    case EFFSC_GKR: return POL_GKR;
    default: return POL_EQFR;
    }
}
int sem_of(const effsc_prover* p) {
    if (p->order == EFFSC_LSB) return SEM_LSB;
    return p->kind == EFFSC_COEF ? SEM_MSB_FLOOR : SEM_MSB_PAD;
}
size_t next_pow2(size_t n) { size_t r = 1; while (r < n) r <<= 1; return r; }
bool is_pow2(size_t n) { return n && !(n & (n - 1)); }
// Blocks for `work` items, at least `per_thread` items per thread and at
// most max_grid().  The cheap Multilinear rounds take four per thread (fewer
// blocks: fewer grid-ticket atomics and partials for the last block to sum,
// which dominate their mid-size rounds); the other provers keep one, their
// mid-size rounds want every thread (measured).
bool cheap_pol(int pol) { return pol == POL_ML; }
int grid_for(u64 work, u64 per_thread = 1) {
    u64 g = (work + per_thread * KERNEL_TPB - 1) / (per_thread * KERNEL_TPB);
    if (g < 1) g = 1;
    u64 mg = (u64)max_grid();
    return (int)(g < mg ? g : mg);
}

// GkrProver passes whose b-variable pairs run in groups sharing one W_b entry
// (k_gkr.cu): from GKR_RUNS_MIN pairs on, a grid of a quarter of the threads
// gives each lane a run of four.  At most one wave of two blocks per SM (the
// kernels' residency): k = 12 measured 0.731 -> 0.694 ms per proof.
constexpr u64 GKR_RUNS_MIN = 1ULL << 17;
int gkr_grid(u64 pairs, bool runs) {
    return std::min<int>(grid_for(pairs, runs && pairs >= GKR_RUNS_MIN ? 4 : 1), (max_grid() / 8) * 2);
}

int alloc_buf(effsc_prover* P, Buf& b, size_t cap, bool ext) {
    b.cap = cap;
    b.ext = ext;
    b.owned = true;
    size_t bytes = (cap ? cap : 1) * sizeof(u64);
    for (int c = 0; c < (ext ? 3 : 1); c++) {
        cudaError_t e = cudaMallocAsync((void**)&b.p[c], bytes, P->ctx->stream);
        if (e != cudaSuccess) return fail(EFFSC_OOM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    }
    return EFFSC_OK;
}
void free_buf(effsc_prover* P, Buf& b) {
    if (!b.owned) return;
    for (int c = 0; c < 3; c++)
        if (b.p[c]) { cudaFreeAsync(b.p[c], P->ctx->stream); b.p[c] = nullptr; }
}

// Pick (or allocate) the output buffer of a fold: never bufs[0] (the input
// table), in place when allowed and the type matches.
int out_buffer(effsc_prover* P, Table& T, bool ext, size_t size, bool inplace_ok, int* out_idx) {
    if (inplace_ok && T.cur != 0 && T.bufs[T.cur].ext == ext && T.bufs[T.cur].cap >= size) { *out_idx = T.cur; return EFFSC_OK; }
    for (size_t i = 1; i < T.bufs.size(); i++)
        if ((int)i != T.cur && T.bufs[i].ext == ext && T.bufs[i].cap >= size) { *out_idx = (int)i; return EFFSC_OK; }
    Buf b;
    TRY(alloc_buf(P, b, size, ext));
    T.bufs.push_back(b);
    *out_idx = (int)T.bufs.size() - 1;
    return EFFSC_OK;
}

RoundArgs base_args(effsc_prover* P) {
    RoundArgs a;
    memset(&a, 0, sizeof a);
    a.partials = P->partials;
    a.counter = P->counter;
    a.status = P->status;
    a.result = P->d_res;
    return a;
}
void set_in(RoundArgs& a, int slot, const Table& T) {
    const Buf& b = T.bufs[T.cur];
    for (int c = 0; c < 3; c++) a.t[slot].in[c] = b.p[c];
}
void set_out(RoundArgs& a, int slot, const Buf& b) {
    for (int c = 0; c < 3; c++) a.t[slot].out[c] = b.p[c];
}

// A round's challenge: absent (round 0), a host value, or a device slot.
struct Chal {
    bool has = false;
    bool ext = false;
    const u64* dev = nullptr;
    u64 v[3] = {0, 0, 0};
};
void put_chal(RoundArgs& a, const Chal& ch) {
    a.chal_ptr = ch.dev;
    for (int c = 0; c < 3; c++) a.chal[c] = ch.v[c];
}

int check_launch(bool ok, const char* what) {
    if (!ok) return fail(EFFSC_UNSUPPORTED, "no kernel instantiated for %s", what);
    g_launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(EFFSC_CUDA_ERROR, "%s launch: %s", what, cudaGetErrorString(e));
    return EFFSC_OK;
}

// Per-launch timing for measurement: CUDA events recorded on the launch
// stream right before and after each kernel, with the kernel's algorithmic
// bytes (every table element it must read plus every element it writes).
struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
    uint64_t bytes;
};
thread_local bool g_prof = false;
thread_local bool g_capturing = false;
thread_local std::vector<ProfRec> g_prof_recs;

template <class F>
int timed_launch(cudaStream_t s, const char* name, uint64_t bytes, F fn) {
    bool prof = g_prof && !g_capturing;
    cudaEvent_t a = nullptr, b = nullptr;
    if (prof) { cudaEventCreate(&a); cudaEventRecord(a, s); }
    bool ok = fn();
    if (prof) {
        cudaEventCreate(&b);
        cudaEventRecord(b, s);
        g_prof_recs.push_back({name, a, b, bytes});
    }
    return check_launch(ok, name);
}
inline uint64_t wbytes(bool ext) { return ext ? 24 : 8; }
// Rounds with at least this many quadruples use the TMA-staged kernel.
const u64 TMA_MIN_QUADS = 1ULL << 15;

// Fold table `ti` of P (kernel slot `slot`) with semantics `sem`.
int fold_table(effsc_prover* P, int ti, int sem, const Chal& ch, bool ech, bool dry) {
    Table& T = P->t[ti];
    size_t L = T.len;
    if (L <= 1) return EFFSC_OK;       // fold of a length-0/1 table is a no-op
    size_t nl = sem == SEM_MSB_PAD ? next_pow2(L) / 2 : L / 2;
    bool out_ext = T.ext || ech;
    int bi;
    TRY(out_buffer(P, T, out_ext, nl, sem != SEM_LSB, &bi));
    if (!dry) {
        RoundArgs a = base_args(P);
        put_chal(a, ch);
        a.L = L;
        set_in(a, 0, T);
        set_out(a, 0, T.bufs[bi]);
        u64 work = sem == SEM_MSB_PAD ? next_pow2(L) / 2 : L / 2;
        uint64_t bytes = L * wbytes(T.ext) + nl * wbytes(out_ext);
        TRY(timed_launch(P->ctx->stream, "fold", bytes, [&] { return launch_fold(sem, T.ext, ech, a, 0, grid_for(work), P->ctx->stream); }));
    }
    T.cur = bi;
    T.len = nl;
    T.ext = out_ext;
    return EFFSC_OK;
}

u32 mask_of(const effsc_prover* P, const int* idx, int n) {
    u32 m = 0;
    for (int i = 0; i < n; i++)
        if (P->t[idx[i]].ext) m |= 1u << i;
    return m;
}

// One round of Multilinear / InnerProduct / Coefficient provers
// (src/provers/multilinear.rs:58-67, multilinear_lsb.rs:180-189,
// inner_product.rs:61-113, inner_product_lsb.rs:156-164,
// coefficient.rs:272-294, coefficient_lsb.rs:180-203).
// One round of a CoefficientProver[LSB] with a declarative evaluator
// (src/provers/coefficient.rs:272-294, coefficient_lsb.rs:180-203): fold
// every column with the challenge (MSB floor or LSB pairs), then evaluate the
// term program over the pairs.
int round_expr(effsc_prover* P, const Chal& ch, const TxIO& tx, bool dry) {
    const int sem = sem_of(P), nt = P->ntab;
    if (ch.has && P->t[0].len > 1) {
        bool ech = ch.ext;
        for (int i = 0; i < nt; i++) ech |= P->t[i].ext;
        for (int i = 0; i < nt; i++) TRY(fold_table(P, i, sem, ch, ech, dry));
    }
    RoundArgs a = base_args(P);
    a.tx = tx;
    const size_t L = P->t[0].len;
    for (int i = 0; i < nt; i++) set_in(a, i, P->t[i]);
    a.L = L;
    uint64_t bytes = 0;
    for (int i = 0; i < nt; i++) bytes += L * wbytes(P->t[i].ext);
    if (!dry) TRY(timed_launch(P->ctx->stream, "expr_evaluate", bytes, [&] {
        return launch_expr_eval(sem, a, P->prog, grid_for(L > 1 ? L / 2 : 1), P->ctx->stream);
    }));
    return EFFSC_OK;
}

int round_std(effsc_prover* P, const Chal& ch, const TxIO& tx, bool dry) {
    if (P->expr) return round_expr(P, ch, tx, dry);
    // the device protocol needs only the wire, not the legacy pair: the
    // degree-3 evaluator then skips h(1)
    const int pol = (pol_of(P) == POL_C3 && tx.tx) ? POL_C3W : pol_of(P), sem = sem_of(P), nt = P->ntab;
    int idx[3] = {0, 1, 2};
    size_t L = P->t[0].len;
    RoundArgs a = base_args(P);
    a.tx = tx;
    put_chal(a, ch);
    if (ch.has && L > 1) {
        bool any_ext = false;
        for (int i = 0; i < nt; i++) any_ext |= P->t[i].ext;
        bool ech = ch.ext || any_ext;
        bool fusable = sem == SEM_MSB_PAD ? (is_pow2(L) && L >= 4) : (L % 4 == 0 && L >= 4);
        if (fusable) {
            u32 mask = mask_of(P, idx, nt);
            int bi[3];
            for (int i = 0; i < nt; i++) {
                Table& T = P->t[i];
                TRY(out_buffer(P, T, T.ext || ech, L / 2, sem != SEM_LSB, &bi[i]));
                set_in(a, i, T);
                set_out(a, i, T.bufs[bi[i]]);
            }
            a.L = L;
            uint64_t bytes = 0;
            for (int i = 0; i < nt; i++) bytes += L * wbytes(P->t[i].ext) + (L / 2) * wbytes(P->t[i].ext || ech);
            const char* nm = mask ? "fused_round_fp3" : (ech ? "fused_round_fp_to_fp3" : "fused_round_fp");
            // large power-of-two rounds: the TMA-staged kernel (LSB also
            // stores the folded pairs with 16-byte stores)
            const u64 Q = L / 4;
            bool tma = pol == POL_IP && (sem == SEM_MSB_PAD || sem == SEM_LSB) && is_pow2(L) && Q >= TMA_MIN_QUADS &&
                       Q % KERNEL_TPB == 0;
            for (int i = 0; i < nt; i++) tma &= !P->t[i].bufs[P->t[i].cur].host;
            for (int i = 0; i < nt && tma; i++)
                for (int c = 0; c < 3; c++) {
                    if (c < (P->t[i].ext ? 3 : 1)) tma &= ((uintptr_t)a.t[i].in[c] % 16) == 0;
                    if (sem == SEM_LSB && a.t[i].out[c]) tma &= ((uintptr_t)a.t[i].out[c] % 16) == 0;
                }
            if (tma) {
                u32 ntiles = (u32)(Q / KERNEL_TPB);
                int g = std::min<int>((int)ntiles, (max_grid() / 8) * fused_tma_blocks_per_sm());
                if (!dry) TRY(timed_launch(P->ctx->stream, nm, bytes, [&] { return launch_fused_tma(pol, sem, mask, ech, a, ntiles, g, P->ctx->stream); }));
            } else {
                if (!dry) TRY(timed_launch(P->ctx->stream, nm, bytes, [&] { return launch_fused(pol, sem, mask, ech, a, grid_for(L / 4, cheap_pol(pol) ? 4 : 1), P->ctx->stream); }));
            }
            for (int i = 0; i < nt; i++) {
                Table& T = P->t[i];
                T.cur = bi[i];
                T.len = L / 2;
                T.ext = T.ext || ech;
            }
            return EFFSC_OK;
        }
        for (int i = 0; i < nt; i++) TRY(fold_table(P, i, sem, ch, ech, dry));
        L = P->t[0].len;
    } else if (!ch.has && P->kind == EFFSC_IP && P->order == EFFSC_LSB && L >= 3 && (L & 1)) {
        // compute_lsb indexes a[i + 1] past the end for odd lengths
        // (src/provers/inner_product_lsb.rs:66-73): the reference panics.
        return fail(EFFSC_PANIC, "InnerProductProverLSB round 0 on odd length %zu (the reference panics)", L);
    }
    // evaluate on the current tables
    for (int i = 0; i < nt; i++) set_in(a, i, P->t[i]);
    a.L = L;
    u64 work = sem == SEM_MSB_PAD ? (L > 1 ? next_pow2(L) / 2 : 1) : sem == SEM_MSB_FLOOR ? L / 2 : (L + 1) / 2;
    uint64_t bytes = 0;
    for (int i = 0; i < nt; i++) bytes += L * wbytes(P->t[i].ext);
    if (!dry) TRY(timed_launch(P->ctx->stream, "evaluate", bytes, [&] { return launch_eval(pol, sem, mask_of(P, idx, nt), a, grid_for(work, cheap_pol(pol) ? 4 : 1), P->ctx->stream); }));
    return EFFSC_OK;
}

// Whether rounds r .. num_rounds-1 of effsc_prove can run in the one-block
// tail kernel: Multilinear / InnerProduct (MSB, or LSB on a bit-reversed
// layout), equal power-of-two tables that
// fit in shared memory, challenges in device memory, and every round still
// folding to at least two entries (the length-1 cases stay on the per-round
// path).
// The tail kernels' policy for a prover: Multilinear and InnerProduct; -1
// for the others.  (A tail for the Coefficient product evaluator of degree 3
// over Fp3 measured slower than its per-round kernels: n = 24, 16 rounds,
// 1.557 ms with the cluster tail from 2^14 entries, 1.533 ms with the
// one-block tail from 2048, 1.519 ms without -- one SM folding and
// evaluating 1024 triple products per round costs more than the launch it
// saves.)
int tail_pol(const effsc_prover* P) {
    if (P->kind == EFFSC_ML || P->kind == EFFSC_IP) return pol_of(P);
    return -1;
}

bool tail_ok(const effsc_prover* P, size_t r, size_t num_rounds, const Chal& ch) {
    if (tail_pol(P) < 0 || !P->tail_len) return false;
    if (r >= num_rounds || (ch.has && !ch.dev)) return false;
    const size_t L = P->t[0].len;
    for (int i = 1; i < P->ntab; i++)
        if (P->t[i].len != L) return false;
    if (!is_pow2(L)) return false;
    const int fw = P->field == EFFSC_FP3 ? 3 : 1;
    const size_t lim = std::min<size_t>(P->tail_len, (size_t)tail_max_len(tail_pol(P), fw, TAIL_SMEM_CAP));
    if (L > lim) return false;
    const size_t rounds = num_rounds - r, folds = rounds - (ch.has ? 0 : 1);
    return folds < 63 && (L >> folds) >= 2;
}

// cluster tail: the same tables up to tail_cluster_max() times one block's
// capacity, entered mid-proof (a challenge to fold with), with at least
// log2(CS) + 1 rounds left; *cs_log = log2(CS), CS = L / capacity.
bool cluster_tail_ok(const effsc_prover* P, size_t r, size_t num_rounds, const Chal& ch, u32* cs_log) {
    // the tail's provers, MSB (the slices need MSB pairs)
    if (tail_pol(P) < 0 || P->order != EFFSC_MSB || !P->tail_len) return false;
    if (r >= num_rounds || !ch.has || !ch.dev) return false;
    const size_t L = P->t[0].len;
    for (int i = 1; i < P->ntab; i++)
        if (P->t[i].len != L) return false;
    if (!is_pow2(L) || L > P->tail_len) return false;
    const int fw = P->field == EFFSC_FP3 ? 3 : 1;
    const size_t cap = (size_t)tail_max_len(tail_pol(P), fw, TAIL_SMEM_CAP);
    if (L <= cap) return false;
    const size_t cs = L / cap, csmax = tail_cluster_max();
    if (cs > csmax || cs < 2 || cap < 32 * cs) return false;   // slices of whole 16-entry groups
    u32 lg = 0;
    while (((size_t)1 << lg) < cs) lg++;
    const size_t rounds = num_rounds - r;
    if (rounds < lg + 1 || rounds >= 63 || (L >> rounds) < 2) return false;
    *cs_log = lg;
    return true;
}

// Rounds r .. r + *nr - 1 of effsc_prove in one cooperative launch
// (k_persist.cu): an InnerProduct prover over Fp3 with equal power-of-two
// device tables of at most persist_len entries, already folded once (so in
// buffers of the prover's own), and a challenge in device memory; the rounds run while the tables are larger than the one-block
// tail takes (at least two rounds, else the per-round kernels stay).
bool persist_ok(const effsc_prover* P, size_t r, size_t num_rounds, const Chal& ch, size_t* nr) {
    if (P->kind != EFFSC_IP || P->field != EFFSC_FP3 || !P->persist_len || !ch.has || !ch.dev) return false;
    const size_t L = P->t[0].len;
    if (P->t[1].len != L || !is_pow2(L) || L < 4 || L > P->persist_len) return false;
    // folds write the current buffers (MSB in place, LSB ping-pong), so
    // never the caller's input tables (bufs[0]); 16-byte loads and stores
    for (int i = 0; i < 2; i++) {
        const Table& T = P->t[i];
        if (!T.ext || T.cur == 0 || T.bufs[T.cur].host) return false;
        for (int c = 0; c < 3; c++)
            if ((uintptr_t)T.bufs[T.cur].p[c] & 15) return false;
    }
    size_t lim = P->tail_len ? std::min<size_t>(P->tail_len, (size_t)tail_max_len(POL_IP, 3, TAIL_SMEM_CAP)) : 0;
    // MSB: stop where the cluster tail takes over (tables of up to
    // tail_cluster_max() times the one-block capacity)
    if (lim && P->order == EFFSC_MSB && tail_cluster_max() >= 2) {
        const size_t cl = lim * tail_cluster_max();
        if (cl <= P->tail_len) lim = cl;
    }
    size_t n = 0, l = L;
    while (r + n < num_rounds && l > lim && l >= 4) { n++; l >>= 1; }
    *nr = n;
    return n >= 2 && persist_max_grid(P->order == EFFSC_LSB) > 0;
}

int do_persist(effsc_prover* P, size_t r, size_t nr, const Chal& ch, size_t hook_len, bool dry) {
    const bool lsb = P->order == EFFSC_LSB;
    const size_t L = P->t[0].len;
    cudaStream_t s = P->ctx->stream;
    if (!P->d_bar) {
        CK(cudaMallocAsync((void**)&P->d_bar, 2 * sizeof(u32), s));
        CK(cudaMemsetAsync(P->d_bar, 0, 2 * sizeof(u32), s));
    }
    PersistArgs p;
    memset(&p, 0, sizeof p);
    int other[2] = {0, 0};
    for (int i = 0; i < 2; i++) {
        Table& T = P->t[i];
        // LSB ping-pongs between the current buffer and another of L / 2
        if (lsb) TRY(out_buffer(P, T, true, L / 2, false, &other[i]));
        for (int c = 0; c < 3; c++) {
            p.buf[0][i][c] = T.bufs[T.cur].p[c];
            p.buf[1][i][c] = lsb ? T.bufs[other[i]].p[c] : nullptr;
        }
    }
    uint64_t bytes = 0;
    for (size_t k = 0; k < nr; k++) bytes += 2 * ((L >> k) * 24 + (L >> (k + 1)) * 24);
    if (!dry) {
        RoundArgs a = base_args(P);
        a.tx.tx = P->d_tx;
        a.tx.hook = P->d_hook;
        a.tx.hook_len = (u32)hook_len;
        p.nrounds = (u32)nr;
        p.L0 = L;
        p.chal_in = ch.dev;
        p.proof_wire = P->d_wire + r * 6;
        p.proof_chal = P->d_chals + 3 * r;
        p.bar = P->d_bar;
        const u64 want = (L / 4 + KERNEL_TPB - 1) / KERNEL_TPB;
        const int cap = std::min(persist_max_grid(lsb), max_grid());
        const int g = (int)std::max<u64>(1, std::min<u64>(want, (u64)cap));
        TRY(timed_launch(s, "ip_rounds_persistent", bytes, [&] { return launch_ip_persist(lsb, a, p, g, s); }));
    }
    for (int i = 0; i < 2; i++) {
        Table& T = P->t[i];
        if (lsb && (nr & 1)) T.cur = other[i];
        T.len = L >> nr;
    }
    P->rounds += nr;
    return EFFSC_OK;
}

// fin: the tail also runs the runner's finalize (the last challenge's fold)
// and writes the tables' first entries to `first` (the proof read-back).
int do_tail(effsc_prover* P, size_t r, size_t num_rounds, const Chal& ch, const TxIO& tx, bool dry, u32 cs_log = 0,
            bool fin = false, u64* first = nullptr) {
    const int pol = tail_pol(P), fw = P->field == EFFSC_FP3 ? 3 : 1, nt = P->ntab;
    const size_t L = P->t[0].len, rounds = num_rounds - r, folds = rounds - (ch.has ? 0 : 1) + (fin ? 1 : 0);
    TailArgs ta;
    memset(&ta, 0, sizeof ta);
    ta.L = L;
    ta.nrounds = (u32)rounds;
    ta.first_fold = ch.has ? 1 : 0;
    ta.chal_in = ch.dev;
    ta.tx = tx.tx;
    ta.hook = tx.hook;
    ta.hook_len = tx.hook_len;
    ta.proof_wire = tx.proof_wire;
    ta.proof_chal = tx.proof_chal;
    ta.final_fold = fin ? 1 : 0;
    ta.first_out = first;
    ta.lsb = P->order == EFFSC_LSB ? 1 : 0;
    const bool out_ext = fw == 3;
    int bi[3] = {0, 0, 0};
    uint64_t bytes = 0;
    for (int i = 0; i < nt; i++) {
        Table& T = P->t[i];
        for (int c = 0; c < 3; c++) ta.in[i][c] = T.bufs[T.cur].p[c];
        if (T.ext) ta.in_ext |= 1u << i;
        bytes += L * wbytes(T.ext);
        if (folds) {
            TRY(out_buffer(P, T, out_ext, L >> folds, true, &bi[i]));
            for (int c = 0; c < 3; c++) ta.out[i][c] = T.bufs[bi[i]].p[c];
            bytes += (L >> folds) * wbytes(out_ext);
        }
    }
    if (!dry) {
        if (cs_log) TRY(timed_launch(P->ctx->stream, "tail_cluster", bytes, [&] { return launch_tail_cluster(pol, fw, ta, cs_log, P->ctx->stream); }));
        else TRY(timed_launch(P->ctx->stream, "tail", bytes, [&] { return launch_tail(pol, fw, nullptr, &ta, 1, L, P->ctx->stream); }));
    }
    if (folds)
        for (int i = 0; i < nt; i++) {
            Table& T = P->t[i];
            T.cur = bi[i];
            T.len = L >> folds;
            T.ext = out_ext;
        }
    return EFFSC_OK;
}

// effsc_prove of a Coefficient prover with the degree-3 product evaluator
// over three device tables of one power-of-two length (table 0 in Fp or Fp3,
// tables 1-2 in Fp, Fp3 challenges): rounds 0 and 1 from one pass (15
// triple-product sums), round 2 with the folds by r0 and r1 from a second
// (k_coef01.cu).  Leaves the state the per-round path leaves after round 2.
constexpr size_t COEF3_MIN_LEN = (size_t)1 << 12;
bool coef3_first_ok(const effsc_prover* P, size_t num_rounds) {
    if (!P->fuse_first || P->kind != EFFSC_COEF || P->expr || P->ntab != 3 || P->field != EFFSC_FP3) return false;
    if (num_rounds < 3) return false;
    const size_t L = P->t[0].len;
    if (!is_pow2(L) || L < COEF3_MIN_LEN) return false;
    for (int i = 0; i < 3; i++) {
        const Table& T = P->t[i];
        if (T.len != L || T.cur != 0 || T.bufs[0].host) return false;
        if (i > 0 && T.ext) return false;
    }
    return true;
}

int do_coef3_first(effsc_prover* P, const TxIO& tx0, const TxIO& tx2, const u64* chals, bool dry) {
    const size_t L = P->t[0].len;
    const bool lsb = P->order == EFFSC_LSB, e0 = P->t[0].ext;
    RoundArgs a = base_args(P);
    a.tx = tx0;
    a.L = L;
    for (int i = 0; i < 3; i++) set_in(a, i, P->t[i]);
    // partials of 48 words per block: max_grid() / 4 blocks at most
    const int g1 = std::min<int>(grid_for(L), max_grid() / 4);   // a quadruple per group thread
    if (!dry) TRY(timed_launch(P->ctx->stream, "coef_rounds_0_1", (uint64_t)L * (e0 ? 40 : 24), [&] {
        return launch_c3_r01(lsb, e0, a, g1, P->ctx->stream);
    }));
    int bi[3];
    for (int i = 0; i < 3; i++) TRY(out_buffer(P, P->t[i], true, L / 4, true, &bi[i]));
    RoundArgs b = base_args(P);
    b.tx = tx2;
    b.L = L;
    b.chal_ptr = chals;
    b.chal2_ptr = chals + 3;
    for (int i = 0; i < 3; i++) {
        set_in(b, i, P->t[i]);
        set_out(b, i, P->t[i].bufs[bi[i]]);
    }
    if (!dry) TRY(timed_launch(P->ctx->stream, "coef_round_2_double_fold", (uint64_t)L * (e0 ? 40 : 24) + 18 * (uint64_t)L, [&] {
        return launch_c3_r2x(lsb, e0, b, grid_for(L / 8), P->ctx->stream);
    }));
    for (int i = 0; i < 3; i++) {
        Table& T = P->t[i];
        T.cur = bi[i];
        T.len = L / 4;
        T.ext = true;
    }
    return EFFSC_OK;
}


// effsc_prove of an InnerProduct prover (MSB or LSB) over Fp3 challenges whose base
// tables are powers of two: rounds 0 and 1 from one pass, round 2 (with the
// folds by r0 and r1) from a second (k_ip01.cu).  Leaves the state the
// per-round path leaves after round 2.
bool fuse_first_ok(const effsc_prover* P, size_t num_rounds) {
    if (!P->fuse_first || P->kind != EFFSC_IP || P->field != EFFSC_FP3) return false;
    if (num_rounds < 3) return false;
    const size_t L = P->t[0].len;
    if (P->t[1].len != L || !is_pow2(L) || L < 8 || P->t[0].ext || P->t[1].ext) return false;
    if (P->t[0].cur != 0 || P->t[1].cur != 0) return false;
    // the LSB pass reads pairs of entries as one 16-byte load
    if (P->order == EFFSC_LSB)
        for (int i = 0; i < 2; i++)
            if (((uintptr_t)P->t[i].bufs[0].p[0] & 15) != 0) return false;
    Chal none;
    return !tail_ok(P, 0, num_rounds, none);
}

// Rounds 0-3 in two passes (k_ip012.cu) from num_vars = 14 on (below, the
// one-block tail takes the proof within a few rounds): leaves the state the
// per-round path leaves after round 3.
constexpr size_t FUSE3_MIN_LEN = 1 << 14;
bool fuse3_ok(const effsc_prover* P, size_t num_rounds) {
    if (P->fuse_first < 2 || num_rounds < 4 || !fuse_first_ok(P, num_rounds)) return false;
    return P->t[0].len >= FUSE3_MIN_LEN;
}

// The mirror of host tables for the two-pass start: both tables in host
// memory, unfolded, and 16 L bytes free on the device beside the Fp3 tables
// the second pass writes (decided once per prover, when no mirror exists).
bool mirror_ok(effsc_prover* P, size_t L) {
    for (int i = 0; i < 2; i++) {
        const Table& T = P->t[i];
        if (T.cur != 0 || !T.bufs[0].host || T.ext) return false;
    }
    if (P->mirror < 0) {
        size_t fr = 0, tot = 0;
        const size_t need = 2 * L * sizeof(u64) + 2 * (L / 8) * 24 + ((size_t)1 << 28);
        P->mirror = cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr >= need ? 1 : 0;
        cudaGetLastError();
    }
    return P->mirror == 1;
}

// Pinned host tables of an MSB prover with room on the device: upload them
// in UPLOAD_CHUNKS chunks of whole octets (octets m in [c O/C, (c+1) O/C),
// one 2-D copy per table: eight rows of O/C entries at stride O) on a copy
// stream, and run the first pass on each chunk as soon as it has arrived,
// carrying the 26 sums from chunk to chunk; the last chunk's launch
// finalises rounds 0-2.  The copy engines then set the pace and all but the
// last chunk's pass hide behind the transfer.
bool upload_chunks_ok(const effsc_prover* P, size_t L) {
    if (P->order != EFFSC_MSB) return false;
    const size_t O = L / 8;
    if (O % ((size_t)UPLOAD_CHUNKS * ip012_tile_octets()) != 0) return false;
    for (int i = 0; i < 2; i++) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, P->t[i].bufs[0].p[0]) != cudaSuccess) { cudaGetLastError(); return false; }
        if (at.type != cudaMemoryTypeHost) return false;   // pageable: the kernel reads it in place
    }
    return true;
}

int chunked_first_pass(effsc_prover* P, RoundArgs a, const int* mi, bool dry) {
    cudaStream_t s = P->ctx->stream;
    const size_t L = P->t[0].len, O = L / 8, CW = O / UPLOAD_CHUNKS;
    if (!P->copy_stream) CK(cudaStreamCreateWithFlags(&P->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : P->chunk_ev)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!P->d_acc) CK(cudaMallocAsync((void**)&P->d_acc, 32 * sizeof(u64), s));
    if (dry) return EFFSC_OK;
    // the copies start after the stream's earlier work (the buffers' allocation)
    CK(cudaEventRecord(P->chunk_ev[UPLOAD_CHUNKS], s));
    CK(cudaStreamWaitEvent(P->copy_stream, P->chunk_ev[UPLOAD_CHUNKS], 0));
    const u32 ct = (u32)(CW / ip012_tile_octets());
    const int g = std::min<int>((int)ct, (max_grid() / 8) * 2);
    for (int i = 0; i < 2; i++) a.t[i].in[0] = P->t[i].bufs[mi[i]].p[0];
    a.acc = P->d_acc;
    for (int c = 0; c < UPLOAD_CHUNKS; c++) {
        for (int i = 0; i < 2; i++)
            CK(cudaMemcpy2DAsync(P->t[i].bufs[mi[i]].p[0] + c * CW, O * sizeof(u64), P->t[i].bufs[0].p[0] + c * CW,
                                 O * sizeof(u64), CW * sizeof(u64), 8, cudaMemcpyHostToDevice, P->copy_stream));
        CK(cudaEventRecord(P->chunk_ev[c], P->copy_stream));
        CK(cudaStreamWaitEvent(s, P->chunk_ev[c], 0));
        a.tile0 = (u32)c * ct;
        a.acc_mode = c == 0 ? ACC_FIRST : c == UPLOAD_CHUNKS - 1 ? ACC_LAST : ACC_MID;
        TRY(timed_launch(s, "ip_rounds_0_2_chunked", 16 * (uint64_t)CW * 8, [&] { return launch_ip012_staged(false, a, ct, g, s); }));
    }
    return EFFSC_OK;
}

int do_fuse3(effsc_prover* P, const TxIO& tx0, const TxIO& tx3, const u64* chals, bool dry) {
    const size_t L = P->t[0].len;
    const bool lsb = P->order == EFFSC_LSB;
    RoundArgs a = base_args(P);
    a.tx = tx0;
    a.L = L;
    for (int i = 0; i < 2; i++) set_in(a, i, P->t[i]);
    // First pass, MSB: staged through shared memory for device tables
    // (16-byte aligned, as the allocator gives).  LSB keeps direct loads: a
    // thread's octet is 64 contiguous bytes, and reading those from a staged
    // tile conflicts on the shared-memory banks (measured slower: 0.51 against
    // 0.40 ms at n = 26).  A block takes 128 octets per step; one wave of two
    // blocks per SM at most (the partials hold 32 words for each).  The
    // second pass reads directly in both orders (staged, MSB measured 0.447
    // against 0.36 ms at n = 26).
    bool staged = !lsb;
    for (int i = 0; i < 2; i++) {
        const Buf& b0 = P->t[i].bufs[0];
        staged &= !b0.host && ((uintptr_t)b0.p[0] & 15) == 0;
    }
    const u32 nt1 = (u32)((L / 8) / ip012_tile_octets());
    staged &= nt1 >= 1 && (L / 8) % ip012_tile_octets() == 0;
    const int two_per_sm = (max_grid() / 8) * 2;
    const int g1 = staged ? std::min<int>((int)nt1, two_per_sm) : std::min<int>(grid_for(L / 8, 2), two_per_sm);
    // Tables in host memory: when the device has room, the first pass also
    // copies them into device buffers (the mirror), so they cross the host
    // link once and the second pass reads HBM.
    int mi[2] = {-1, -1};
    if (mirror_ok(P, L))
        for (int i = 0; i < 2; i++) {
            TRY(out_buffer(P, P->t[i], false, L, false, &mi[i]));
            a.t[i].out[0] = P->t[i].bufs[mi[i]].p[0];
        }
    if (mi[0] >= 0 && upload_chunks_ok(P, L)) {
        TRY(chunked_first_pass(P, a, mi, dry));
    } else if (!dry) {
        TRY(timed_launch(P->ctx->stream, mi[0] >= 0 ? "ip_rounds_0_2_from_host" : "ip_rounds_0_2", 16 * (uint64_t)L, [&] {
            if (mi[0] >= 0) return launch_ip012_mirror(lsb, a, g1, P->ctx->stream);
            return staged ? launch_ip012_staged(lsb, a, nt1, g1, P->ctx->stream) : launch_ip012(lsb, a, g1, P->ctx->stream);
        }));
    }
    if (mi[0] >= 0)
        for (int i = 0; i < 2; i++) P->t[i].cur = mi[i];
    int bi[2];
    for (int i = 0; i < 2; i++) TRY(out_buffer(P, P->t[i], true, L / 8, true, &bi[i]));
    RoundArgs b = base_args(P);
    b.tx = tx3;
    b.L = L;
    b.chal_ptr = chals;
    for (int i = 0; i < 2; i++) {
        set_in(b, i, P->t[i]);
        set_out(b, i, P->t[i].bufs[bi[i]]);
    }
    // one wave (two blocks per SM, the kernel's residency): n = 26 measured
    // 0.369 against 0.377 ms (MSB) and 0.350 against 0.364 ms (LSB) for four
    // waves of blocks
    if (!dry) TRY(timed_launch(P->ctx->stream, "ip_round_3_triple_fold", 16 * (uint64_t)L + 6 * (uint64_t)L, [&] {
        return launch_ip3x(lsb, b, std::min<int>(grid_for(L / 16), two_per_sm), P->ctx->stream);
    }));
    for (int i = 0; i < 2; i++) {
        Table& T = P->t[i];
        T.cur = bi[i];
        T.len = L / 8;
        T.ext = true;
    }
    return EFFSC_OK;
}

int do_fuse_first(effsc_prover* P, const TxIO& tx0, const TxIO& tx2, const u64* chals, bool dry) {
    const size_t L = P->t[0].len;
    RoundArgs a = base_args(P);
    a.tx = tx0;
    a.L = L;
    for (int i = 0; i < 2; i++) set_in(a, i, P->t[i]);
    if (!dry) TRY(timed_launch(P->ctx->stream, "ip_rounds_0_1", 16 * (uint64_t)L, [&] { return launch_ip01(P->order == EFFSC_LSB, a, grid_for(L / 4), P->ctx->stream); }));
    int bi[2];
    for (int i = 0; i < 2; i++) TRY(out_buffer(P, P->t[i], true, L / 4, true, &bi[i]));
    RoundArgs b = base_args(P);
    b.tx = tx2;
    b.L = L;
    b.chal_ptr = chals;
    b.chal2_ptr = chals + 3;
    for (int i = 0; i < 2; i++) {
        set_in(b, i, P->t[i]);
        set_out(b, i, P->t[i].bufs[bi[i]]);
    }
    if (!dry) TRY(timed_launch(P->ctx->stream, "ip_round_2_double_fold", 16 * (uint64_t)L + 12 * (uint64_t)L, [&] { return launch_ip2x(P->order == EFFSC_LSB, b, grid_for(L / 8), P->ctx->stream); }));
    for (int i = 0; i < 2; i++) {
        Table& T = P->t[i];
        T.cur = bi[i];
        T.len = L / 4;
        T.ext = true;
    }
    return EFFSC_OK;
}

// effsc_prove of an MSB Multilinear prover over a power-of-two base table:
// rounds 0 and 1 from one pass (quarter sums), round 2 with the folds by r0
// and r1 from a second (ml01.cuh).  Leaves the state the per-round path
// leaves after round 2.
bool ml_first_ok(const effsc_prover* P, size_t num_rounds) {
    if (!P->fuse_first || P->kind != EFFSC_ML || P->order != EFFSC_MSB || num_rounds < 3) return false;
    const Table& T = P->t[0];
    if (T.ext || T.cur != 0 || !is_pow2(T.len) || T.len < 8) return false;
    Chal none;
    if (tail_ok(P, 0, num_rounds, none)) return false;
    // a table the cluster tail takes from round 1 on runs faster that way
    // (measured: n = 18 over Fp)
    const int fw = P->field == EFFSC_FP3 ? 3 : 1;
    const size_t cap = (size_t)tail_max_len(POL_ML, fw, TAIL_SMEM_CAP) * std::max<u32>(1, tail_cluster_max());
    return T.len > cap || T.len > P->tail_len;
}

int do_ml_first(effsc_prover* P, const TxIO& tx0, const TxIO& tx2, const u64* chals, bool dry) {
    Table& T = P->t[0];
    const size_t L = T.len;
    const bool ech = P->field == EFFSC_FP3;
    RoundArgs a = base_args(P);
    a.tx = tx0;
    a.L = L;
    set_in(a, 0, T);
    if (!dry) TRY(timed_launch(P->ctx->stream, "ml_rounds_0_1", 6 * (uint64_t)L, [&] { return launch_ml01(a, grid_for(L / 4, 4), P->ctx->stream); }));
    int bi;
    TRY(out_buffer(P, T, ech, L / 4, true, &bi));
    RoundArgs b = base_args(P);
    b.tx = tx2;
    b.L = L;
    b.chal_ptr = chals;
    b.chal2_ptr = chals + 3;
    set_in(b, 0, T);
    set_out(b, 0, T.bufs[bi]);
    if (!dry) TRY(timed_launch(P->ctx->stream, "ml_round_2_double_fold", 8 * (uint64_t)L + (L / 4) * wbytes(ech), [&] { return launch_ml2x(ech, b, grid_for(L / 8, 4), P->ctx->stream); }));
    T.cur = bi;
    T.len = L / 4;
    T.ext = ech;
    return EFFSC_OK;
}

// GkrProver tail: from round r on, the four tables in one block's shared
// memory (k_gkr_tail.cu) -- the remaining rounds, the finalize and the
// read-back entries in one launch.  Leaves the state the per-round path and
// finalize leave.
bool gkr_tail_ok(const effsc_prover* P, size_t r, size_t num_rounds, const Chal& ch) {
    if (P->kind != EFFSC_GKR || !P->tail_len || r >= num_rounds || (ch.has && !ch.dev)) return false;
    if (num_rounds - r > ((size_t)1 << 20) || P->t[0].len > P->tail_len) return false;
    size_t tot = 0;
    for (int i = 0; i < 4; i++) {
        if (!is_pow2(P->t[i].len)) return false;
        tot += P->t[i].len;
    }
    const size_t fw = P->field == EFFSC_FP3 ? 3 : 1;
    return tot <= TAIL_SMEM_CAP / (8 * fw);
}

int do_gkr_tail(effsc_prover* P, size_t r, size_t num_rounds, const Chal& ch, const TxIO& tx, bool dry, u64* first) {
    const int fw = P->field == EFFSC_FP3 ? 3 : 1;
    const size_t k = P->v_l;
    GkrTailArgs ta;
    memset(&ta, 0, sizeof ta);
    ta.nrounds = (u32)(num_rounds - r);
    ta.r0 = (u32)r;
    ta.k = (u32)k;
    ta.first_fold = ch.has ? 1 : 0;
    ta.final_fold = 1;
    ta.chal_in = ch.dev;
    ta.tx = tx.tx;
    ta.hook = tx.hook;
    ta.hook_len = tx.hook_len;
    ta.proof_wire = tx.proof_wire;
    ta.proof_chal = tx.proof_chal;
    ta.first_out = first;
    // the lengths the folds leave: each round (but a first one without a
    // challenge) and the finalize fold the gate tables and the witness table
    // of the variable just bound
    size_t len[4], tot = 0;
    for (int i = 0; i < 4; i++) len[i] = P->t[i].len;
    auto fold_len = [&](size_t var) {
        for (int i : {0, 1, var < k ? 2 : 3})
            if (len[i] >= 2) len[i] >>= 1;
    };
    for (size_t j = ch.has ? 0 : 1; j < num_rounds - r; j++) fold_len(r + j - 1);
    fold_len(num_rounds - 1);
    uint64_t bytes = 0;
    int bi[4];
    for (int i = 0; i < 4; i++) {
        Table& T = P->t[i];
        for (int c = 0; c < 3; c++) ta.in[i][c] = T.bufs[T.cur].p[c];
        if (T.ext) ta.in_ext |= 1u << i;
        ta.len[i] = T.len;
        tot += T.len;
        bytes += T.len * wbytes(T.ext) + len[i] * wbytes(fw == 3);
        TRY(out_buffer(P, T, fw == 3, len[i], true, &bi[i]));
        for (int c = 0; c < 3; c++) ta.out[i][c] = T.bufs[bi[i]].p[c];
    }
    if (!dry) TRY(timed_launch(P->ctx->stream, "gkr_tail", bytes, [&] { return launch_gkr_tail(fw, ta, 8 * fw * tot, P->ctx->stream); }));
    for (int i = 0; i < 4; i++) {
        Table& T = P->t[i];
        T.cur = bi[i];
        T.len = len[i];
        T.ext = fw == 3;
    }
    P->rounds = num_rounds;
    return EFFSC_OK;
}

// effsc_prove of a GkrProver with k >= 3 over base add, mult and witness:
// rounds 0 and 1 from one pass, round 2 with the folds of add and mult by r0
// and r1 from a second (k_gkr.cu).  Leaves the state the per-round path
// leaves after round 2: add and mult folded twice, W_b folded by r0 and r1.
bool gkr_first_ok(const effsc_prover* P, size_t num_rounds) {
    if (!P->fuse_first || P->kind != EFFSC_GKR || P->rounds != 0 || num_rounds < 3 || P->v_l < 3) return false;
    Chal none;
    if (gkr_tail_ok(P, 0, num_rounds, none)) return false;
    const size_t n = (size_t)1 << P->v_l;
    for (int i = 0; i < 4; i++) {
        const Table& T = P->t[i];
        if (T.ext || T.cur != 0 || T.len != (i < 2 ? n * n : n)) return false;
    }
    return true;
}

int do_gkr_first(effsc_prover* P, const TxIO& tx0, const TxIO& tx2, const u64* chals, bool dry) {
    const size_t N = P->t[0].len, n = P->t[2].len;
    const bool ech = P->field == EFFSC_FP3;
    cudaStream_t s = P->ctx->stream;
    RoundArgs a = base_args(P);
    a.tx = tx0;
    a.L = N;
    a.m_shift = (u32)P->v_l;
    for (int i = 0; i < 4; i++) set_in(a, i, P->t[i]);
    // large passes: runs of quadruples at three blocks per SM (k_gkr_r01_runs)
    const int g3 = (int)std::min<u64>((u64)(max_grid() / 8) * 3, (N / 4 + KERNEL_TPB - 1) / KERNEL_TPB);
    const u64 nw3 = (u64)g3 * KERNEL_TPB / 32;
    const u64 run3 = std::min<u64>(std::min<u64>((N / 4) / (32 * nw3), 16), (u64)n >> 5);
    if (!dry) TRY(timed_launch(s, "gkr_rounds_0_1", 16 * (uint64_t)N + 16 * (uint64_t)n, [&] {
        return run3 >= 2 ? launch_gkr01_runs(a, g3, s) : launch_gkr01(a, gkr_grid(N / 4, true), s);
    }));
    // W_b folded by r0, then r1 (the per-round path folds it as rounds 1 and 2 start)
    for (int r = 0; r < 2; r++) {
        Chal c;
        c.has = true;
        c.ext = ech;
        c.dev = chals + 3 * r;
        TRY(fold_table(P, 2, SEM_MSB_PAD, c, ech, dry));
    }
    int bi[2];
    for (int i = 0; i < 2; i++) TRY(out_buffer(P, P->t[i], ech, N / 4, true, &bi[i]));
    RoundArgs b = base_args(P);
    b.tx = tx2;
    b.L = N;
    b.m_shift = (u32)P->v_l;
    b.chal_ptr = chals;
    b.chal2_ptr = chals + 3;
    for (int i = 0; i < 4; i++) set_in(b, i, P->t[i]);
    for (int i = 0; i < 2; i++) set_out(b, i, P->t[i].bufs[bi[i]]);
    if (!dry) TRY(timed_launch(s, "gkr_round_2_double_fold", 16 * (uint64_t)N + 2 * (N / 4) * wbytes(ech), [&] { return launch_gkr2x(ech, b, gkr_grid(N / 8, true), s); }));
    for (int i = 0; i < 2; i++) {
        Table& T = P->t[i];
        T.cur = bi[i];
        T.len = N / 4;
        T.ext = ech;
    }
    P->rounds = 3;
    return EFFSC_OK;
}

// effsc_prove of an EqFactored prover whose run covers the whole left phase
// (num_rounds >= v_l >= 2) with eq_l small enough for the one-block tail: the
// left rounds are InnerProduct rounds on (eq_l, S), S[a] = sum_b eq_r[b]
// p[a m + b] (k_eqf.cu).  Leaves the state the per-round path leaves after
// round v_l - 1: p folded by r_0 .. r_{v_l-2}, eq_l of length 2, eq_r as is.
bool eqf_fast_ok(const effsc_prover* P, size_t num_rounds) {
    if (!P->fuse_first || P->kind != EFFSC_EQF || P->rounds != 0) return false;
    const size_t vl = P->v_l;
    if (vl < 2 || num_rounds < vl) return false;
    const Table &p = P->t[0], &el = P->t[1], &er = P->t[2];
    if (p.cur != 0 || el.cur != 0 || er.cur != 0) return false;
    if (p.len != ((size_t)1 << P->v) || el.len != ((size_t)1 << vl) || er.len != ((size_t)1 << (P->v - vl))) return false;
    const int fw = P->field == EFFSC_FP3 ? 3 : 1;
    return el.len <= (size_t)tail_max_len(POL_IP, fw, TAIL_SMEM_CAP);
}

int do_eqf_left(effsc_prover* P, const TxIO& tx, bool dry) {
    const int fw = P->field == EFFSC_FP3 ? 3 : 1;
    const size_t vl = P->v_l;
    Table &p = P->t[0], &el = P->t[1], &er = P->t[2];
    const u64 m = er.len, rows = el.len;
    const u64 rows2 = (u64)1 << (vl - 1), Lc = p.len >> (vl - 1);
    const u64 splits = rows2 < 64 ? rows2 : 64;
    cudaStream_t s = P->ctx->stream;
    const size_t need = 3 * rows + 3 * rows2 + 3 * splits * Lc;
    if (P->eqf_cap < need) {
        if (P->eqf_scratch) CK(cudaFreeAsync(P->eqf_scratch, s));
        P->eqf_scratch = nullptr;
        CK(cudaMallocAsync((void**)&P->eqf_scratch, need * sizeof(u64), s));
        P->eqf_cap = need;
    }
    u64* S = P->eqf_scratch;
    u64* Ew = S + 3 * rows;
    u64* part = Ew + 3 * rows2;
    const bool out_ext = fw == 3;
    int bp, be;
    TRY(out_buffer(P, p, p.ext || out_ext, Lc, true, &bp));
    TRY(out_buffer(P, el, el.ext || out_ext, 2, true, &be));
    if (!dry) {
        Tab3 tp, ter, te;
        for (int c = 0; c < 3; c++) {
            tp.c[c] = p.bufs[p.cur].p[c];
            ter.c[c] = er.bufs[er.cur].p[c];
        }
        u64* s1 = fw == 3 ? S + rows : nullptr;
        u64* s2 = fw == 3 ? S + 2 * rows : nullptr;
        const uint64_t b1 = p.len * wbytes(p.ext) + m * wbytes(er.ext) + rows * wbytes(out_ext);
        TRY(timed_launch(s, "eqf_inner_sums", b1, [&] {
            launch_eqf_inner(er.ext, p.ext, tp, ter, m, rows, S, s1, s2, s);
            return true;
        }));
        TailArgs ta;
        memset(&ta, 0, sizeof ta);
        for (int c = 0; c < 3; c++) ta.in[0][c] = el.bufs[el.cur].p[c];
        if (el.ext) ta.in_ext |= 1u;
        ta.in[1][0] = S;
        ta.in[1][1] = s1;
        ta.in[1][2] = s2;
        if (fw == 3) ta.in_ext |= 2u;
        for (int c = 0; c < 3; c++) ta.out[0][c] = el.bufs[be].p[c];
        ta.out[1][0] = S;
        ta.out[1][1] = s1;
        ta.out[1][2] = s2;
        ta.L = rows;
        ta.nrounds = (u32)vl;
        ta.first_fold = 0;
        ta.tx = tx.tx;
        ta.hook = tx.hook;
        ta.hook_len = tx.hook_len;
        ta.proof_wire = tx.proof_wire;
        ta.proof_chal = tx.proof_chal;
        TRY(timed_launch(s, "tail", 2 * rows * wbytes(out_ext), [&] { return launch_tail(POL_IP, fw, nullptr, &ta, 1, rows, s); }));
        // eq weights of r_0 .. r_{v_l-2} (MSB order), then the weighted row sum of p
        launch_build_eq(P->d_chals, (u32)(vl - 1), fw == 3, Ew, Ew + rows2, Ew + 2 * rows2, s);
        g_launches++;
        te.c[0] = Ew;
        te.c[1] = fw == 3 ? Ew + rows2 : nullptr;
        te.c[2] = fw == 3 ? Ew + 2 * rows2 : nullptr;
        const Buf& ob = p.bufs[bp];
        const uint64_t b2 = p.len * wbytes(p.ext) + Lc * wbytes(p.ext || out_ext) + 2 * splits * Lc * 24;
        TRY(timed_launch(s, "eqf_fold_left", b2, [&] {
            launch_eqf_fold_rows(fw == 3, p.ext, tp, te, Lc, rows2, splits, part, fw, ob.p[0], ob.p[1], ob.p[2], s);
            return true;
        }));
        g_launches++;   // the sum over row groups
    }
    p.cur = bp;
    p.len = Lc;
    p.ext = p.ext || out_ext;
    el.cur = be;
    el.len = 2;
    el.ext = el.ext || out_ext;
    P->rounds = vl;
    return EFFSC_OK;
}

// One round of EqFactoredProver (src/provers/eq_factored.rs:249-270).
int round_eqf(effsc_prover* P, const Chal& ch, const TxIO& tx, bool dry) {
    Table &p = P->t[0], &el = P->t[1], &er = P->t[2];
    RoundArgs a = base_args(P);
    a.tx = tx;
    put_chal(a, ch);
    const size_t j = P->rounds;
    const bool left = j < P->v_l;
    bool done = false;
    if (ch.has) {
        size_t prev_var = P->rounds - 1;   // wraps like the reference's release build
        bool ech = ch.ext || p.ext || el.ext || er.ext;
        size_t L = p.len;
        if (left && prev_var < P->v_l && is_pow2(L) && L >= 4) {
            // fold eq_l, then fold p fused with the left-phase evaluation
            TRY(fold_table(P, 1, SEM_MSB_PAD, ch, ech, dry));
            int bi;
            TRY(out_buffer(P, p, p.ext || ech, L / 2, true, &bi));
            set_in(a, 0, p);
            set_out(a, 0, p.bufs[bi]);
            set_in(a, 1, el);
            set_in(a, 2, er);
            a.L = L;
            a.el_len = el.len;
            a.m_shift = (u32)__builtin_ctzll(er.len);
            u32 mask = (p.ext ? 1u : 0u) | (el.ext ? 2u : 0u);
            uint64_t bytes = L * wbytes(p.ext) + (L / 2) * wbytes(p.ext || ech) + el.len * wbytes(el.ext) + er.len * wbytes(er.ext);
            if (!dry) TRY(timed_launch(P->ctx->stream, "eqf_left_fused", bytes, [&] { return launch_eqf_left(true, mask, ech, a, grid_for(L / 4), P->ctx->stream); }));
            p.cur = bi;
            p.len = L / 2;
            p.ext = p.ext || ech;
            done = true;
        } else if (!left && prev_var >= P->v_l && is_pow2(L) && L >= 4 && er.len == L) {
            int idx[2] = {2, 0};
            u32 mask = mask_of(P, idx, 2);
            int bi_e, bi_p;
            TRY(out_buffer(P, er, er.ext || ech, L / 2, true, &bi_e));
            TRY(out_buffer(P, p, p.ext || ech, L / 2, true, &bi_p));
            set_in(a, 0, er);
            set_out(a, 0, er.bufs[bi_e]);
            set_in(a, 1, p);
            set_out(a, 1, p.bufs[bi_p]);
            const Buf& sb = el.bufs[el.cur];
            for (int c = 0; c < 3; c++) a.scalar[c] = sb.p[c];
            a.L = L;
            uint64_t bytes = L * (wbytes(er.ext) + wbytes(p.ext)) + (L / 2) * (wbytes(er.ext || ech) + wbytes(p.ext || ech));
            if (!dry) TRY(timed_launch(P->ctx->stream, "eqf_right_fused", bytes, [&] { return launch_fused(POL_EQFR, SEM_MSB_PAD, mask, ech, a, grid_for(L / 4), P->ctx->stream); }));
            er.cur = bi_e; er.len = L / 2; er.ext = er.ext || ech;
            p.cur = bi_p; p.len = L / 2; p.ext = p.ext || ech;
            done = true;
        } else {
            TRY(fold_table(P, 0, SEM_MSB_PAD, ch, ech, dry));
            TRY(fold_table(P, prev_var < P->v_l ? 1 : 2, SEM_MSB_PAD, ch, ech, dry));
        }
    }
    if (!done) {
        if (left) {
            // src/provers/eq_factored.rs:139-172
            set_in(a, 0, p);
            set_in(a, 1, el);
            set_in(a, 2, er);
            a.L = p.len;
            a.el_len = el.len;
            a.m_shift = (u32)__builtin_ctzll(er.len);
            u32 mask = (p.ext ? 1u : 0u) | (el.ext ? 2u : 0u);
            uint64_t bytes = p.len * wbytes(p.ext) + el.len * wbytes(el.ext) + er.len * wbytes(er.ext);
            if (!dry) TRY(timed_launch(P->ctx->stream, "eqf_left_evaluate", bytes, [&] { return launch_eqf_left(false, mask, false, a, grid_for(p.len / 2), P->ctx->stream); }));
        } else {
            // src/provers/eq_factored.rs:178-209
            int idx[2] = {2, 0};
            set_in(a, 0, er);
            set_in(a, 1, p);
            const Buf& sb = el.bufs[el.cur];
            for (int c = 0; c < 3; c++) a.scalar[c] = sb.p[c];
            a.L = p.len;
            u64 work = p.len > 1 ? p.len / 2 : 1;
            uint64_t bytes = p.len * (wbytes(p.ext) + wbytes(er.ext));
            if (!dry) TRY(timed_launch(P->ctx->stream, "eqf_right_evaluate", bytes, [&] { return launch_eval(POL_EQFR, SEM_MSB_PAD, mask_of(P, idx, 2), a, grid_for(work), P->ctx->stream); }));
        }
    }
    P->rounds++;
    return EFFSC_OK;
}

// A kernel that gave up a bounded wait leaves a code in the status word.
int check_status(effsc_prover* P) {
    volatile u32* st = (volatile u32*)(P->h_res + 15);
    u32 v = *st;
    if (!v) return EFFSC_OK;
    *st = 0;
    cudaMemsetAsync(P->counter, 0, sizeof(u32), P->ctx->stream);
    if (P->d_bar) cudaMemsetAsync(P->d_bar, 0, sizeof(u32), P->ctx->stream);
    return fail(EFFSC_TIMEOUT, "a round kernel timed out waiting for its staged loads or grid barrier (status %u)", v);
}

// One round of GkrProver (src/provers/gkr.rs:105-190) on the compact witness
// tables (k_gkr.cu): fold W_b when the variable just bound is a b variable
// (the first k), else W_c; fold add and mult fused with the evaluation.
int round_gkr(effsc_prover* P, const Chal& ch, const TxIO& tx, bool dry) {
    Table &A = P->t[0], &M = P->t[1], &WB = P->t[2], &WC = P->t[3];
    RoundArgs a = base_args(P);
    a.tx = tx;
    put_chal(a, ch);
    a.m_shift = (u32)P->v_l;
    bool fused = false;
    bool ech = false;
    if (ch.has) {
        const size_t prev_var = P->rounds - 1;   // wraps like the reference's release build
        ech = ch.ext || A.ext || M.ext || WB.ext || WC.ext;
        TRY(fold_table(P, prev_var < P->v_l ? 2 : 3, SEM_MSB_PAD, ch, ech, dry));
        const size_t L = A.len;
        if (is_pow2(L) && L >= 4) {
            fused = true;
        } else {
            TRY(fold_table(P, 0, SEM_MSB_PAD, ch, ech, dry));
            TRY(fold_table(P, 1, SEM_MSB_PAD, ch, ech, dry));
        }
    }
    const size_t L = A.len;
    for (int i = 0; i < 4; i++) set_in(a, i, P->t[i]);
    a.L = L;
    int bi[2] = {0, 0};
    const bool ea = A.ext;
    if (fused)
        for (int i = 0; i < 2; i++) {
            TRY(out_buffer(P, P->t[i], P->t[i].ext || ech, L / 2, true, &bi[i]));
            set_out(a, i, P->t[i].bufs[bi[i]]);
        }
    const bool ewb = WB.ext, ewc = WC.ext;
    const u64 Ln = fused ? L / 2 : L;
    uint64_t bytes = 2 * (L * wbytes(ea) + (fused ? (L / 2) * wbytes(ea || ech) : 0)) +
                     WB.len * wbytes(ewb) + WC.len * wbytes(ewc);
    if (!dry) TRY(timed_launch(P->ctx->stream, fused ? "gkr_fused_round" : "gkr_evaluate", bytes, [&] {
        const bool runs = !ewc && P->v_l < 64 && ((u64)1 << P->v_l) < Ln;   // a b variable, W_c in the base field
        return launch_gkr(fused, ea, ewb, ewc, fused && (ech || ea), a, gkr_grid(Ln > 1 ? Ln / 2 : 1, runs), P->ctx->stream);
    }));
    if (fused)
        for (int i = 0; i < 2; i++) {
            Table& T = P->t[i];
            T.cur = bi[i];
            T.len = L / 2;
            T.ext = T.ext || ech;
        }
    P->rounds++;
    return EFFSC_OK;
}

int do_round(effsc_prover* P, const Chal& ch, const TxIO& tx, bool dry) {
    if (P->kind == EFFSC_GKR) return round_gkr(P, ch, tx, dry);
    return P->kind == EFFSC_EQF ? round_eqf(P, ch, tx, dry) : round_std(P, ch, tx, dry);
}

// SumcheckProver::finalize of every prover.
int do_finalize(effsc_prover* P, const Chal& ch, bool dry) {
    if (P->kind == EFFSC_EQF) {
        // src/provers/eq_factored.rs:272-280 (last_var = v - 1, wrapping)
        bool ech = ch.ext || P->t[0].ext || P->t[1].ext || P->t[2].ext;
        size_t last_var = P->v - 1;
        TRY(fold_table(P, 0, SEM_MSB_PAD, ch, ech, dry));
        TRY(fold_table(P, last_var < P->v_l ? 1 : 2, SEM_MSB_PAD, ch, ech, dry));
        return EFFSC_OK;
    }
    if (P->kind == EFFSC_GKR) {
        // src/provers/gkr.rs:193-198 folds all four tables; with the compact
        // witness only the table of the variable being bound changes
        bool ech = ch.ext;
        for (int i = 0; i < 4; i++) ech |= P->t[i].ext;
        const size_t last_var = P->rounds - 1;
        TRY(fold_table(P, 0, SEM_MSB_PAD, ch, ech, dry));
        TRY(fold_table(P, 1, SEM_MSB_PAD, ch, ech, dry));
        TRY(fold_table(P, last_var < P->v_l ? 2 : 3, SEM_MSB_PAD, ch, ech, dry));
        return EFFSC_OK;
    }
    bool ech = ch.ext;
    for (int i = 0; i < P->ntab; i++) ech |= P->t[i].ext;
    for (int i = 0; i < P->ntab; i++) TRY(fold_table(P, i, sem_of(P), ch, ech, dry));
    return EFFSC_OK;
}

// Entry 0 of each table's current buffer, gathered on the device by
// effsc_prove (k_gather_first) so that the final value needs no extra copy.
thread_local const u64* g_first = nullptr;
constexpr size_t TX_OUT_WORDS = (sizeof(DevTranscript) + 7) / 8;

int read_first(effsc_prover* P, int ti, HF* out) {
    if (g_first) {
        *out = hf(g_first[3 * ti], g_first[3 * ti + 1], g_first[3 * ti + 2]);
        return EFFSC_OK;
    }
    Table& T = P->t[ti];
    const Buf& b = T.bufs[T.cur];
    u64 w[3] = {0, 0, 0};
    for (int c = 0; c < (T.ext ? 3 : 1); c++)
        CK(cudaMemcpyAsync(&w[c], b.p[c], sizeof(u64), cudaMemcpyDefault, P->ctx->stream));
    CK(cudaStreamSynchronize(P->ctx->stream));
    *out = hf(w[0], w[1], w[2]);
    return EFFSC_OK;
}

// SumcheckProver::final_value of every prover.
// final_value of a declarative evaluator (src/provers/coefficient.rs:300-329,
// coefficient_lsb.rs:215-236): the evaluator on (singleton, 0) pairs, then
// h(0) + h(1).  A lone pairwise table's singleton is returned as is (MSB: any
// degree; LSB: degree 1).  A tablewise table's odd row is an empty slice in
// the reference, so a term reading it panics there.
int final_value_expr(effsc_prover* P, HF* out) {
    const ExprProgram& g = P->prog;
    const int nt = P->ntab;
    const bool lone = P->n_pairwise == 1 && P->tw_cols == 0 && P->t[0].len == 1;
    if (lone && (P->order == EFFSC_MSB || g.degree == 1)) return read_first(P, 0, out);
    HF even[4];
    for (int c = 0; c < nt; c++) {
        even[c] = hf(0);
        if (P->t[c].len == 1) TRY(read_first(P, c, &even[c]));
    }
    HF coef[4] = {hf(0), hf(0), hf(0), hf(0)};
    for (u32 t = 0; t < g.nterms; t++) {
        const ExprTerm& T = g.t[t];
        HF p = hf(T.k[0], T.k[1], T.k[2]);
        for (u32 f = 0; f < T.nf; f++) {
            const int col = T.f[f] >> 1, odd = T.f[f] & 1;
            // a tablewise table's pair is (its row, []) when it holds one
            // row and ([], []) otherwise: indexing an empty row panics
            if (((P->tw_cols >> col) & 1) && (odd || P->t[col].len != 1))
                return fail(EFFSC_PANIC, "final_value: the evaluator reads an empty tablewise row (the odd row, "
                                         "or any row of a table not folded to one row); the reference panics");
            p = hf_mul(p, odd ? hf(0) : even[col]);
        }
        coef[T.coeff] = hf_add(coef[T.coeff], p);
    }
    HF h1 = hf(0);
    for (u32 j = 0; j <= g.degree && j < 4; j++) h1 = hf_add(h1, coef[j]);
    *out = hf_add(coef[0], h1);
    return EFFSC_OK;
}

int final_value(effsc_prover* P, HF* out) {
    *out = hf(0);
    switch (P->kind) {
    case EFFSC_ML:   // src/provers/multilinear.rs:74-79
        if (P->t[0].len == 1) TRY(read_first(P, 0, out));
        return EFFSC_OK;
    case EFFSC_IP: { // src/provers/inner_product.rs:120-126
        if (P->t[0].len != 1) return EFFSC_OK;
        HF a, b;
        TRY(read_first(P, 0, &a));
        TRY(read_first(P, 1, &b));
        *out = hf_mul(a, b);
        return EFFSC_OK;
    }
    case EFFSC_COEF: { // src/provers/coefficient.rs:300-329: h(0) + h(1) of the
        // product evaluator on (singleton, 0) pairs = product of the singletons
        if (P->expr) return final_value_expr(P, out);
        if (P->ntab == 1 && P->t[0].len == 1) return read_first(P, 0, out);
        HF acc = hf(1);
        for (int i = 0; i < P->ntab; i++) {
            HF x = hf(0);
            if (P->t[i].len == 1) TRY(read_first(P, i, &x));
            acc = hf_mul(acc, x);
        }
        // coefficients c(x) = prod (x_i - x x_i): h(0) = prod x_i, h(1) = 0
        *out = acc;
        return EFFSC_OK;
    }
    case EFFSC_GKR: { // src/provers/gkr.rs:200-208
        if (P->t[0].len != 1) return EFFSC_OK;
        HF a, m, wb, wc;
        TRY(read_first(P, 0, &a));
        TRY(read_first(P, 1, &m));
        TRY(read_first(P, 2, &wb));
        TRY(read_first(P, 3, &wc));
        *out = hf_add(hf_mul(a, hf_add(wb, wc)), hf_mul(m, hf_mul(wb, wc)));
        return EFFSC_OK;
    }
    default: {       // src/provers/eq_factored.rs:282-288
        if (P->t[0].len != 1) return EFFSC_OK;
        HF pv, a, b;
        TRY(read_first(P, 0, &pv));
        TRY(read_first(P, 1, &a));
        TRY(read_first(P, 2, &b));
        *out = hf_mul(hf_mul(pv, a), b);
        return EFFSC_OK;
    }
    }
}

int prover_common_init(effsc_prover* P) {
    cudaStream_t s = P->ctx->stream;
    CK(cudaMallocAsync((void**)&P->partials, (size_t)max_grid() * 12 * sizeof(u64), s));
    CK(cudaMallocAsync((void**)&P->counter, 2 * sizeof(u32), s));
    CK(cudaMemsetAsync(P->counter, 0, 2 * sizeof(u32), s));
    P->h_res = (u64*)pinned_get(P->ctx, 16 * sizeof(u64));
    if (!P->h_res) return fail(EFFSC_OOM, "pinned result block");
    CK(cudaHostGetDevicePointer((void**)&P->d_res, P->h_res, 0));
    memset(P->h_res, 0, 16 * sizeof(u64));
    // word 15 of the mapped result block: kernel status (0 = ok)
    P->status = (u32*)(P->d_res + 15);
    return EFFSC_OK;
}

// Upload one host table (AoS, ncomp words per element) into bufs[0].
int upload_table(effsc_prover* P, Table& T, const uint64_t* host, size_t len, int ncomp, int repr) {
    cudaStream_t s = P->ctx->stream;
    Buf b;
    if (ncomp == 1) {
        TRY(alloc_buf(P, b, len, false));
        if (len) CK(cudaMemcpyAsync(b.p[0], host, len * sizeof(u64), cudaMemcpyHostToDevice, s));
        if (repr == EFFSC_MONTGOMERY && len) {
            launch_split_aos(b.p[0], len, 1, b.p[0], nullptr, nullptr, 1, nullptr, s);
            g_launches++;
        }
    } else {
        TRY(alloc_buf(P, b, len, true));
        u64* stage = nullptr;
        u32* flag = nullptr;
        CK(cudaMallocAsync((void**)&stage, (len ? len : 1) * 3 * sizeof(u64), s));
        CK(cudaMallocAsync((void**)&flag, sizeof(u32), s));
        CK(cudaMemsetAsync(flag, 0, sizeof(u32), s));
        if (len) {
            CK(cudaMemcpyAsync(stage, host, len * 3 * sizeof(u64), cudaMemcpyHostToDevice, s));
            launch_split_aos(stage, len, 3, b.p[0], b.p[1], b.p[2], repr == EFFSC_MONTGOMERY, flag, s);
            g_launches++;
        }
        u32 hflag = 0;
        CK(cudaMemcpyAsync(&hflag, flag, sizeof(u32), cudaMemcpyDeviceToHost, s));
        CK(cudaFreeAsync(stage, s));
        CK(cudaFreeAsync(flag, s));
        CK(cudaStreamSynchronize(s));
        if (!hflag) {
            // every element is embedded (c1 = c2 = 0): keep the base component
            cudaFreeAsync(b.p[1], s);
            cudaFreeAsync(b.p[2], s);
            b.p[1] = b.p[2] = nullptr;
            b.ext = false;
        }
    }
    T.bufs.clear();
    T.bufs.push_back(b);
    T.cur = 0;
    T.len = len;
    T.ext = b.ext;
    return EFFSC_OK;
}

// Make table T an Fp3 table (input buffer replaced by its embedded copy).
int promote(effsc_prover* P, Table& T) {
    if (T.ext) return EFFSC_OK;
    cudaStream_t s = P->ctx->stream;
    Buf nb;
    TRY(alloc_buf(P, nb, T.len, true));
    Buf& ob = T.bufs[T.cur];
    if (T.len) {
        CK(cudaMemcpyAsync(nb.p[0], ob.p[0], T.len * sizeof(u64), cudaMemcpyDefault, s));
        CK(cudaMemsetAsync(nb.p[1], 0, T.len * sizeof(u64), s));
        CK(cudaMemsetAsync(nb.p[2], 0, T.len * sizeof(u64), s));
    }
    for (auto& b : T.bufs) free_buf(P, b);
    T.bufs.clear();
    T.bufs.push_back(nb);
    T.cur = 0;
    T.ext = true;
    return EFFSC_OK;
}

// Keep every table combination on an instantiated kernel: mixed base/Fp3
// tables are promoted except the (Fp3, base, base) CoefficientProver shape
// (eq(r, x) * f * g with base f, g).
int normalize_masks(effsc_prover* P) {
    if (P->kind == EFFSC_GKR) {
        // add and mult share one representation, and so do the two witness
        // tables at the start; each witness table turns Fp3 when its own
        // fold with an Fp3 challenge does (W_c only in the last k rounds)
        if (P->t[2].ext != P->t[3].ext) { TRY(promote(P, P->t[2])); TRY(promote(P, P->t[3])); }
        if (P->t[0].ext != P->t[1].ext) { TRY(promote(P, P->t[0])); TRY(promote(P, P->t[1])); }
        return EFFSC_OK;
    }
    if (P->kind == EFFSC_EQF) {
        if (P->field == EFFSC_FP3 || P->t[0].ext) { TRY(promote(P, P->t[1])); TRY(promote(P, P->t[2])); }
        return EFFSC_OK;
    }
    int nt = P->ntab;
    bool any = false, all = true;
    for (int i = 0; i < nt; i++) { any |= P->t[i].ext; all &= P->t[i].ext; }
    if (!any || all) return EFFSC_OK;
    if (P->kind == EFFSC_COEF && nt == 3 && P->t[0].ext && !P->t[1].ext && !P->t[2].ext) return EFFSC_OK;
    for (int i = 0; i < nt; i++) TRY(promote(P, P->t[i]));
    return EFFSC_OK;
}

void snapshot_initial(effsc_prover* P) {
    for (int i = 0; i < 4; i++) { P->len0[i] = P->t[i].len; P->ext0[i] = P->t[i].ext; }
}

int check_field(int field) {
    if (field != EFFSC_FP && field != EFFSC_FP3) return fail(EFFSC_INVALID_ARG, "field must be EFFSC_FP (1) or EFFSC_FP3 (3)");
    return EFFSC_OK;
}

void release_prover(effsc_prover* P) {
    if (!P) return;
    if (P->ctx) {
        cudaSetDevice(P->ctx->device);
        cudaStreamSynchronize(P->ctx->stream);
        for (int i = 0; i < 4; i++)
            for (auto& b : P->t[i].bufs) free_buf(P, b);
        cudaStream_t s = P->ctx->stream;
        if (P->partials) cudaFreeAsync(P->partials, s);
        if (P->counter) cudaFreeAsync(P->counter, s);
        if (P->d_bar) cudaFreeAsync(P->d_bar, s);
        if (P->d_acc) cudaFreeAsync(P->d_acc, s);
        for (cudaEvent_t& e : P->chunk_ev)
            if (e) { cudaEventDestroy(e); e = nullptr; }
        if (P->copy_stream) { cudaStreamDestroy(P->copy_stream); P->copy_stream = nullptr; }
        if (P->d_tx) cudaFreeAsync(P->d_tx, s);
        if (P->d_hook) cudaFreeAsync(P->d_hook, s);
        if (P->d_wire) cudaFreeAsync(P->d_wire, s);
        if (P->d_chals) cudaFreeAsync(P->d_chals, s);
        if (P->eqf_scratch) cudaFreeAsync(P->eqf_scratch, s);
        if (P->d_first) cudaFreeAsync(P->d_first, s);
        if (P->gexec) cudaGraphExecDestroy(P->gexec);
        cudaStreamSynchronize(s);
    }
    if (P->ctx) {
        pinned_put(P->ctx, P->h_res, 16 * sizeof(u64));
        pinned_put(P->ctx, P->h_out, P->h_out_bytes);
    } else {
        if (P->h_res) cudaFreeHost(P->h_res);
        if (P->h_out) cudaFreeHost(P->h_out);
    }
    delete P;
}

Chal host_chal(const effsc_prover* P, const uint64_t* c) {
    Chal ch;
    ch.has = c != nullptr;
    if (c) {
        HF v = load_elem(c, P->field, P->repr);
        for (int i = 0; i < 3; i++) ch.v[i] = v.c[i];
        ch.ext = hf_is_ext(v);
    }
    return ch;
}

}  // namespace

// Internal accessors used by batch.cu / serve.cu / streams.cu.
const u64* effsc_internal_device_view(int device, const uint64_t* ptr, bool* is_host);
void effsc_internal_tx_state(const effsc_transcript* t, void* out) {
    DevTranscript st = t->st;
    if (t->kind != EFFSC_T_KECCAK) st.deg = 0;   // marks a transcript the device cannot run
    memcpy(out, &st, sizeof st);
}
const u64* effsc_internal_device_view(int device, const uint64_t* ptr, bool* is_host) {
    cudaPointerAttributes at;
    *is_host = false;
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return (const u64*)ptr;
    *is_host = true;
    if (at.type == cudaMemoryTypeHost) return (const u64*)at.devicePointer;
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
    return pageable ? (const u64*)ptr : nullptr;
}
void* effsc_internal_pinned_get(effsc_ctx* c, size_t bytes) { return pinned_get(c, bytes); }
void effsc_internal_pinned_put(effsc_ctx* c, void* p, size_t bytes) { pinned_put(c, p, bytes); }
int effsc_internal_ctx_device(const effsc_ctx* c) { return c->device; }
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c) { return c->stream; }
uint64_t effsc_internal_add_launches(uint64_t k) { g_launches += k; return g_launches; }

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* effsc_last_error(void) { return g_err.c_str(); }
const char* effsc_status_str(int s) {
    switch (s) {
    case EFFSC_OK: return "ok";
    case EFFSC_INVALID_ARG: return "invalid argument";
    case EFFSC_OOM: return "out of device memory";
    case EFFSC_CUDA_ERROR: return "CUDA error";
    case EFFSC_TIMEOUT: return "timeout";
    case EFFSC_UNSUPPORTED: return "unsupported";
    case EFFSC_PANIC: return "the reference panics on this input";
    default: return "unknown status";
    }
}
uint64_t effsc_launch_count(void) { return g_launches; }
void effsc_launch_count_reset(void) { g_launches = 0; }

int effsc_profile_enable(int on) {
    g_prof = on != 0;
    return EFFSC_OK;
}
size_t effsc_profile_count(void) { return g_prof_recs.size(); }
int effsc_profile_get(size_t i, char* name, size_t name_cap, double* ms, uint64_t* bytes) {
    if (i >= g_prof_recs.size()) return fail(EFFSC_INVALID_ARG, "profile record %zu out of range", i);
    ProfRec& r = g_prof_recs[i];
    if (name && name_cap) {
        strncpy(name, r.name.c_str(), name_cap - 1);
        name[name_cap - 1] = 0;
    }
    if (ms) {
        CK(cudaEventSynchronize(r.b));
        float f = 0;
        CK(cudaEventElapsedTime(&f, r.a, r.b));
        *ms = f;
    }
    if (bytes) *bytes = r.bytes;
    return EFFSC_OK;
}
void effsc_profile_clear(void) {
    for (auto& r : g_prof_recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    g_prof_recs.clear();
}

int effsc_diag_mulmod_rate(effsc_ctx* ctx, double* mulmod_per_s, double* fp3_mul_per_s) {
    if (!ctx) return fail(EFFSC_INVALID_ARG, "ctx is NULL");
    CK(cudaSetDevice(ctx->device));
    double a = 0, b = 0;
    if (!diag_mulmod_rate(ctx->stream, &a, &b)) return fail(EFFSC_CUDA_ERROR, "mulmod microbenchmark failed");
    if (mulmod_per_s) *mulmod_per_s = a;
    if (fp3_mul_per_s) *fp3_mul_per_s = b;
    return EFFSC_OK;
}

int effsc_diag_accumulate_rate(effsc_ctx* ctx, double* mac_per_s, double* reduce_per_s) {
    if (!ctx) return fail(EFFSC_INVALID_ARG, "ctx is NULL");
    CK(cudaSetDevice(ctx->device));
    double a = 0, b = 0;
    if (!diag_accumulate_rate(ctx->stream, &a, &b)) return fail(EFFSC_CUDA_ERROR, "accumulate microbenchmark failed");
    if (mac_per_s) *mac_per_s = a;
    if (reduce_per_s) *reduce_per_s = b;
    return EFFSC_OK;
}

int effsc_diag_transcript_latency(effsc_ctx* ctx, double* ns_per_permutation, double* ns_per_round_step) {
    if (!ctx) return fail(EFFSC_INVALID_ARG, "ctx is NULL");
    CK(cudaSetDevice(ctx->device));
    u64* d = nullptr;
    u64 h[3] = {0, 0, 0};
    CK(cudaMallocAsync((void**)&d, sizeof h, ctx->stream));
    launch_diag_transcript(2, d, ctx->stream);        // warm-up
    launch_diag_transcript(1000, d, ctx->stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFreeAsync(d, ctx->stream);
    if (e != cudaSuccess) return fail(EFFSC_CUDA_ERROR, "transcript probe: %s", cudaGetErrorString(e));
    if (ns_per_permutation) *ns_per_permutation = (double)h[0];
    if (ns_per_round_step) *ns_per_round_step = (double)h[1];
    return EFFSC_OK;
}

int effsc_ctx_create(int device, effsc_ctx** out) {
    if (!out) return fail(EFFSC_INVALID_ARG, "out is NULL");
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(EFFSC_INVALID_ARG, "device %d out of range (%d devices)", device, n);
    CK(cudaSetDevice(device));
    effsc_ctx* c = new effsc_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return fail(EFFSC_CUDA_ERROR, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
    c->stream = c->own;
    kernels_init(device);
    tail_cluster_max();   // probe the cluster size once, outside any stream capture
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = c;
    return EFFSC_OK;
}
int effsc_ctx_destroy(effsc_ctx* c) {
    if (!c) return EFFSC_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& kv : c->pin_free) cudaFreeHost(kv.second);
    c->pin_free.clear();
    cudaStreamDestroy(c->own);
    delete c;
    return EFFSC_OK;
}
int effsc_ctx_set_stream(effsc_ctx* c, void* s) {
    if (!c) return fail(EFFSC_INVALID_ARG, "ctx is NULL");
    c->stream = s ? (cudaStream_t)s : c->own;
    return EFFSC_OK;
}
int effsc_ctx_synchronize(effsc_ctx* c) {
    if (!c) return fail(EFFSC_INVALID_ARG, "ctx is NULL");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    return EFFSC_OK;
}

int effsc_prover_create(effsc_ctx* ctx, int kind, int order, int field, int repr, int n_tables,
                        const uint64_t* const* tables, const size_t* lens, const int* ncomp, effsc_prover** out) {
    if (!ctx || !out || !tables || !lens || !ncomp) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (kind != EFFSC_ML && kind != EFFSC_IP && kind != EFFSC_COEF) return fail(EFFSC_INVALID_ARG, "kind must be ML, IP or COEF (use effsc_eqf_create)");
    if (order != EFFSC_MSB && order != EFFSC_LSB) return fail(EFFSC_INVALID_ARG, "order must be MSB or LSB");
    int want = kind == EFFSC_ML ? 1 : kind == EFFSC_IP ? 2 : -1;
    if ((want > 0 && n_tables != want) || n_tables < 1 || n_tables > 3)
        return fail(EFFSC_INVALID_ARG, "wrong number of tables (%d)", n_tables);
    for (int i = 0; i < n_tables; i++) {
        if (ncomp[i] != 1 && ncomp[i] != 3) return fail(EFFSC_INVALID_ARG, "ncomp must be 1 or 3");
        if (ncomp[i] == 3 && field != EFFSC_FP3) return fail(EFFSC_INVALID_ARG, "Fp3 table for an Fp prover");
        if (lens[i] && !tables[i]) return fail(EFFSC_INVALID_ARG, "table %d is NULL", i);
    }
    if (kind == EFFSC_IP && lens[0] != lens[1])
        return fail(EFFSC_PANIC, "a and b must have equal length (%zu != %zu)", lens[0], lens[1]);
    if (kind == EFFSC_COEF)
        for (int i = 1; i < n_tables; i++)
            if (lens[i] != lens[0]) return fail(EFFSC_PANIC, "pairwise tables must have equal length");
    CK(cudaSetDevice(ctx->device));
    effsc_prover* P = new effsc_prover();
    P->ctx = ctx; P->kind = kind; P->order = order; P->field = field; P->repr = repr; P->ntab = n_tables;
    int rc = prover_common_init(P);
    for (int i = 0; i < n_tables && rc == EFFSC_OK; i++) rc = upload_table(P, P->t[i], tables[i], lens[i], ncomp[i], repr);
    if (rc == EFFSC_OK) rc = normalize_masks(P);
    if (rc == EFFSC_OK) { cudaError_t e = cudaStreamSynchronize(ctx->stream); if (e != cudaSuccess) rc = fail(EFFSC_CUDA_ERROR, "upload: %s", cudaGetErrorString(e)); }
    if (rc != EFFSC_OK) { release_prover(P); return rc; }
    snapshot_initial(P);
    *out = P;
    return EFFSC_OK;
}

int effsc_coef_expr_create(effsc_ctx* ctx, int order, int field, int repr, int degree, int n_pairwise,
                           const uint64_t* const* pairwise, const int* pw_ncomp, int n_tablewise,
                           const uint64_t* const* tablewise, const size_t* tw_widths, const int* tw_ncomp,
                           size_t len, const effsc_term* terms, size_t n_terms, effsc_prover** out) {
    if (!ctx || !out || (n_terms && !terms)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (order != EFFSC_MSB && order != EFFSC_LSB) return fail(EFFSC_INVALID_ARG, "order must be MSB or LSB");
    if (degree < 0 || degree > 3) return fail(EFFSC_UNSUPPORTED, "declarative evaluators of degree 0..3 (got %d)", degree);
    if (n_pairwise < 0 || n_tablewise < 0 || (n_pairwise && (!pairwise || !pw_ncomp)) ||
        (n_tablewise && (!tablewise || !tw_widths || !tw_ncomp)))
        return fail(EFFSC_INVALID_ARG, "NULL table arrays");
    size_t ncols = (size_t)n_pairwise;
    for (int i = 0; i < n_tablewise; i++) ncols += tw_widths[i];
    if (ncols < 1 || ncols > 4)
        return fail(EFFSC_UNSUPPORTED, "declarative evaluators read 1..4 columns (pairwise tables plus tablewise "
                                       "columns); got %zu", ncols);
    if (n_terms > (size_t)EXPR_MAX_TERMS) return fail(EFFSC_UNSUPPORTED, "at most %d terms", EXPR_MAX_TERMS);
    ExprProgram prog;
    memset(&prog, 0, sizeof prog);
    prog.nterms = (u32)n_terms;
    prog.degree = (u32)(degree < 1 ? 1 : degree);    // degree 0 sends [h(0)] like degree 1
    prog.ncols = (u32)ncols;
    for (size_t t = 0; t < n_terms; t++) {
        const effsc_term& T = terms[t];
        if ((int)T.coeff > degree || T.n_factors > (u32)EXPR_MAX_FACTORS)
            return fail(EFFSC_INVALID_ARG, "term %zu: coefficient %u or %u factors out of range", t, T.coeff, T.n_factors);
        prog.t[t].coeff = (unsigned char)T.coeff;
        prog.t[t].nf = (unsigned char)T.n_factors;
        for (u32 f = 0; f < T.n_factors; f++) {
            if (T.factors[f] >= 2 * ncols) return fail(EFFSC_INVALID_ARG, "term %zu: factor %u names no column", t, T.factors[f]);
            prog.t[t].f[f] = (unsigned char)T.factors[f];
        }
        const HF k = load_elem(T.k, field, repr);
        for (int c = 0; c < 3; c++) prog.t[t].k[c] = k.c[c];
    }
    for (int i = 0; i < n_pairwise; i++) {
        if (pw_ncomp[i] != 1 && pw_ncomp[i] != 3) return fail(EFFSC_INVALID_ARG, "ncomp must be 1 or 3");
        if (pw_ncomp[i] == 3 && field != EFFSC_FP3) return fail(EFFSC_INVALID_ARG, "Fp3 table for an Fp prover");
        if (len && !pairwise[i]) return fail(EFFSC_INVALID_ARG, "pairwise table %d is NULL", i);
    }
    for (int i = 0; i < n_tablewise; i++) {
        if (tw_ncomp[i] != 1 && tw_ncomp[i] != 3) return fail(EFFSC_INVALID_ARG, "ncomp must be 1 or 3");
        if (tw_ncomp[i] == 3 && field != EFFSC_FP3) return fail(EFFSC_INVALID_ARG, "Fp3 table for an Fp prover");
        if (len && tw_widths[i] && !tablewise[i]) return fail(EFFSC_INVALID_ARG, "tablewise table %d is NULL", i);
    }
    CK(cudaSetDevice(ctx->device));
    effsc_prover* P = new effsc_prover();
    P->ctx = ctx; P->kind = EFFSC_COEF; P->order = order; P->field = field; P->repr = repr; P->ntab = (int)ncols;
    P->expr = true;
    P->prog = prog;
    P->n_pairwise = n_pairwise;
    int rc = prover_common_init(P);
    int col = 0;
    for (int i = 0; i < n_pairwise && rc == EFFSC_OK; i++, col++)
        rc = upload_table(P, P->t[col], pairwise[i], len, pw_ncomp[i], repr);
    // a tablewise table is len rows of width w (row-major, ncomp words per
    // element); column c of it becomes its own table of len elements
    for (int i = 0; i < n_tablewise && rc == EFFSC_OK; i++) {
        const size_t w = tw_widths[i], nc = (size_t)tw_ncomp[i];
        std::vector<uint64_t> colbuf(len * nc);
        for (size_t c = 0; c < w && rc == EFFSC_OK; c++, col++) {
            for (size_t r = 0; r < len; r++)
                for (size_t k = 0; k < nc; k++) colbuf[r * nc + k] = tablewise[i][(r * w + c) * nc + k];
            rc = upload_table(P, P->t[col], colbuf.data(), len, (int)nc, repr);
            P->tw_cols |= 1u << col;
            if (rc == EFFSC_OK) { cudaError_t e = cudaStreamSynchronize(ctx->stream); if (e != cudaSuccess) rc = fail(EFFSC_CUDA_ERROR, "upload: %s", cudaGetErrorString(e)); }
        }
    }
    if (rc == EFFSC_OK) { cudaError_t e = cudaStreamSynchronize(ctx->stream); if (e != cudaSuccess) rc = fail(EFFSC_CUDA_ERROR, "upload: %s", cudaGetErrorString(e)); }
    if (rc != EFFSC_OK) { release_prover(P); return rc; }
    snapshot_initial(P);
    *out = P;
    return EFFSC_OK;
}

// A pointer the kernels can read: device memory as is, pinned or registered
// host memory through its device alias, pageable host memory when the GPU
// reads host page tables (cudaDevAttrPageableMemoryAccess); else null.
static const u64* device_view(int device, const uint64_t* ptr, bool* is_host) {
    return effsc_internal_device_view(device, ptr, is_host);
}

// Provers over caller-owned tables read in place (device or host memory).
static int create_in_place(effsc_ctx* ctx, int kind, int order, int field, int n_tables,
                           const uint64_t* const* tables, const size_t* lens, const int* ncomp, bool host,
                           effsc_prover** out) {
    const uint64_t* const* dev_tables = tables;
    if (!ctx || !out || !dev_tables || !lens || !ncomp) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (kind != EFFSC_ML && kind != EFFSC_IP && kind != EFFSC_COEF) return fail(EFFSC_INVALID_ARG, "kind must be ML, IP or COEF");
    int want = kind == EFFSC_ML ? 1 : kind == EFFSC_IP ? 2 : -1;
    if ((want > 0 && n_tables != want) || n_tables < 1 || n_tables > 3) return fail(EFFSC_INVALID_ARG, "wrong number of tables");
    if (kind == EFFSC_IP && lens[0] != lens[1]) return fail(EFFSC_PANIC, "a and b must have equal length");
    if (kind == EFFSC_COEF)
        for (int i = 1; i < n_tables; i++)
            if (lens[i] != lens[0]) return fail(EFFSC_PANIC, "pairwise tables must have equal length");
    CK(cudaSetDevice(ctx->device));
    effsc_prover* P = new effsc_prover();
    P->ctx = ctx; P->kind = kind; P->order = order; P->field = field; P->repr = EFFSC_CANONICAL; P->ntab = n_tables;
    int rc = prover_common_init(P);
    for (int i = 0; i < n_tables && rc == EFFSC_OK; i++) {
        if (ncomp[i] != 1 && ncomp[i] != 3) { rc = fail(EFFSC_INVALID_ARG, "ncomp must be 1 or 3"); break; }
        Buf b;
        b.owned = false;
        b.cap = lens[i];
        b.ext = ncomp[i] == 3;
        b.p[0] = (u64*)dev_tables[i];
        if (host) {
            bool is_host = false;
            const u64* v = device_view(ctx->device, dev_tables[i], &is_host);
            if (!v) { rc = fail(EFFSC_UNSUPPORTED, "table %d: host memory the GPU cannot read (register or pin it)", i); break; }
            b.p[0] = (u64*)v;
            b.host = is_host;
        }
        if (b.ext) { b.p[1] = b.p[0] + lens[i]; b.p[2] = b.p[0] + 2 * lens[i]; }
        Table& T = P->t[i];
        T.bufs.assign(1, b);
        T.cur = 0;
        T.len = lens[i];
        T.ext = b.ext;
    }
    if (rc == EFFSC_OK) {
        bool any = false, all = true;
        for (int i = 0; i < n_tables; i++) { any |= P->t[i].ext; all &= P->t[i].ext; }
        bool coef_eq_shape = kind == EFFSC_COEF && n_tables == 3 && P->t[0].ext && !P->t[1].ext && !P->t[2].ext;
        if (any && !all && !coef_eq_shape) rc = fail(EFFSC_UNSUPPORTED, "mixed base/Fp3 device tables: pass all tables in one field");
    }
    if (rc != EFFSC_OK) { release_prover(P); return rc; }
    snapshot_initial(P);
    *out = P;
    return EFFSC_OK;
}

int effsc_prover_create_device(effsc_ctx* ctx, int kind, int order, int field, int n_tables,
                               const uint64_t* const* dev_tables, const size_t* lens, const int* ncomp,
                               effsc_prover** out) {
    return create_in_place(ctx, kind, order, field, n_tables, dev_tables, lens, ncomp, false, out);
}

int effsc_prover_create_host(effsc_ctx* ctx, int kind, int order, int field, int n_tables,
                             const uint64_t* const* host_tables, const size_t* lens, const int* ncomp,
                             effsc_prover** out) {
    return create_in_place(ctx, kind, order, field, n_tables, host_tables, lens, ncomp, true, out);
}

int effsc_gkr_create(effsc_ctx* ctx, int field, int repr, const uint64_t* add, const uint64_t* mult, const uint64_t* w,
                     size_t n, int ncomp, effsc_prover** out) {
    if (!ctx || !out || !add || !mult || !w) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (ncomp != 1 && ncomp != 3) return fail(EFFSC_INVALID_ARG, "ncomp must be 1 or 3");
    if (!is_pow2(n) || n > ((size_t)1 << 17))
        return fail(EFFSC_UNSUPPORTED, "GkrProver on the device needs |w| a power of two up to 2^17 (got %zu)", n);
    if (ncomp == 3 && field != EFFSC_FP3) return fail(EFFSC_INVALID_ARG, "Fp3 tables for an Fp prover");
    CK(cudaSetDevice(ctx->device));
    effsc_prover* P = new effsc_prover();
    P->ctx = ctx; P->kind = EFFSC_GKR; P->order = EFFSC_MSB; P->field = field; P->repr = repr; P->ntab = 4;
    size_t k = 0;
    while (((size_t)1 << k) < n) k++;
    P->v = 2 * k; P->v_l = k;
    int rc = prover_common_init(P);
    if (rc == EFFSC_OK) rc = upload_table(P, P->t[0], add, n * n, ncomp, repr);
    if (rc == EFFSC_OK) rc = upload_table(P, P->t[1], mult, n * n, ncomp, repr);
    if (rc == EFFSC_OK) rc = upload_table(P, P->t[2], w, n, ncomp, repr);
    if (rc == EFFSC_OK) rc = upload_table(P, P->t[3], w, n, ncomp, repr);
    if (rc == EFFSC_OK) rc = normalize_masks(P);
    if (rc == EFFSC_OK) { cudaError_t e = cudaStreamSynchronize(ctx->stream); if (e != cudaSuccess) rc = fail(EFFSC_CUDA_ERROR, "%s", cudaGetErrorString(e)); }
    if (rc != EFFSC_OK) { release_prover(P); return rc; }
    snapshot_initial(P);
    *out = P;
    return EFFSC_OK;
}

int effsc_gkr_claimed_w_values(effsc_prover* P, uint64_t* out) {
    if (!P || !out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    if (P->kind != EFFSC_GKR) return fail(EFFSC_INVALID_ARG, "not a GkrProver");
    CK(cudaSetDevice(P->ctx->device));
    HF wb = hf(0), wc = hf(0);
    if (P->t[0].len == 1) {
        TRY(read_first(P, 2, &wb));
        TRY(read_first(P, 3, &wc));
    }
    store_elem(out, wb, P->field, P->repr);
    store_elem(out + P->field, wc, P->field, P->repr);
    return EFFSC_OK;
}

int effsc_eqf_create(effsc_ctx* ctx, int field, int repr, const uint64_t* w, size_t num_vars, const uint64_t* pv,
                     size_t p_len, int p_ncomp, effsc_prover** out) {
    if (!ctx || !out || (num_vars && !w) || (p_len && !pv)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (num_vars > 40) return fail(EFFSC_INVALID_ARG, "num_vars too large");
    if (p_ncomp != 1 && p_ncomp != 3) return fail(EFFSC_INVALID_ARG, "p_ncomp must be 1 or 3");
    size_t n = (size_t)1 << num_vars;
    if (p_len > n) return fail(EFFSC_PANIC, "p_evals length %zu exceeds 2^%zu = %zu", p_len, num_vars, n);
    CK(cudaSetDevice(ctx->device));
    effsc_prover* P = new effsc_prover();
    P->ctx = ctx; P->kind = EFFSC_EQF; P->order = EFFSC_MSB; P->field = field; P->repr = repr; P->ntab = 3;
    P->v = num_vars; P->v_l = num_vars / 2;
    int rc = prover_common_init(P);
    cudaStream_t s = ctx->stream;
    // p, zero-padded to 2^v
    if (rc == EFFSC_OK) {
        std::vector<uint64_t> padded;
        const uint64_t* src = pv;
        if (p_len < n) {
            padded.assign(n * (size_t)p_ncomp, 0);
            if (p_len) memcpy(padded.data(), pv, p_len * (size_t)p_ncomp * sizeof(uint64_t));
            if (repr == EFFSC_MONTGOMERY) { /* zero is zero in both encodings */ }
            src = padded.data();
        }
        rc = upload_table(P, P->t[0], src, n, p_ncomp, repr);
    }
    // eq_l, eq_r built on the device from w (src/provers/eq_factored.rs:100-103)
    std::vector<u64> wc(3 * (num_vars ? num_vars : 1), 0);
    bool wext = false;
    for (size_t j = 0; j < num_vars; j++) {
        HF x = load_elem(w + j * (size_t)field, field, repr);
        wc[3 * j] = x.c[0]; wc[3 * j + 1] = x.c[1]; wc[3 * j + 2] = x.c[2];
        wext |= hf_is_ext(x);
    }
    u64* dw = nullptr;
    if (rc == EFFSC_OK) {
        cudaError_t e = cudaMallocAsync((void**)&dw, wc.size() * sizeof(u64), s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dw, wc.data(), wc.size() * sizeof(u64), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) rc = fail(EFFSC_CUDA_ERROR, "w upload: %s", cudaGetErrorString(e));
    }
    for (int h = 0; h < 2 && rc == EFFSC_OK; h++) {
        size_t vv = h == 0 ? P->v_l : num_vars - P->v_l;
        size_t off = h == 0 ? 0 : P->v_l;
        Buf b;
        rc = alloc_buf(P, b, (size_t)1 << vv, wext);
        if (rc != EFFSC_OK) break;
        launch_build_eq(dw + 3 * off, (u32)vv, wext, b.p[0], b.p[1], b.p[2], s);
        g_launches++;
        Table& T = P->t[1 + h];
        T.bufs.assign(1, b);
        T.cur = 0;
        T.len = (size_t)1 << vv;
        T.ext = wext;
    }
    if (dw) cudaFreeAsync(dw, s);
    if (rc == EFFSC_OK) rc = normalize_masks(P);
    if (rc == EFFSC_OK) { cudaError_t e = cudaStreamSynchronize(s); if (e != cudaSuccess) rc = fail(EFFSC_CUDA_ERROR, "%s", cudaGetErrorString(e)); }
    if (rc != EFFSC_OK) { release_prover(P); return rc; }
    snapshot_initial(P);
    *out = P;
    return EFFSC_OK;
}

int effsc_prover_destroy(effsc_prover* p) {
    release_prover(p);
    return EFFSC_OK;
}

int effsc_prover_degree(const effsc_prover* p) { return p ? degree_of(p) : -1; }

int effsc_prover_round(effsc_prover* P, const uint64_t* challenge, uint64_t* out_evals, uint64_t* out_aux) {
    if (!P) return fail(EFFSC_INVALID_ARG, "prover is NULL");
    CK(cudaSetDevice(P->ctx->device));
    Chal ch = host_chal(P, challenge);
    TxIO tx;
    memset(&tx, 0, sizeof tx);
    TRY(do_round(P, ch, tx, false));
    CK(cudaStreamSynchronize(P->ctx->stream));
    TRY(check_status(P));
    int d = degree_of(P);
    const u64* r = P->h_res;
    if (out_evals)
        for (int i = 0; i < d; i++) store_elem(out_evals + (size_t)i * P->field, hf(r[3 * i], r[3 * i + 1], r[3 * i + 2]), P->field, P->repr);
    if (out_aux)
        for (int i = 0; i < 2; i++) {
            const u64* q = r + 3 * d + 3 * i;
            store_elem(out_aux + (size_t)i * P->field, hf(q[0], q[1], q[2]), P->field, P->repr);
        }
    return EFFSC_OK;
}

int effsc_prover_finalize(effsc_prover* P, const uint64_t* challenge) {
    if (!P || !challenge) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(P->ctx->device));
    TRY(do_finalize(P, host_chal(P, challenge), false));
    CK(cudaStreamSynchronize(P->ctx->stream));
    return EFFSC_OK;
}

int effsc_prover_final_value(effsc_prover* P, uint64_t* out) {
    if (!P || !out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(P->ctx->device));
    HF v;
    TRY(final_value(P, &v));
    store_elem(out, v, P->field, P->repr);
    return EFFSC_OK;
}

int effsc_prover_table_len(const effsc_prover* P, int table, size_t* out) {
    if (!P || !out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    int nt = P->kind == EFFSC_EQF ? 3 : P->kind == EFFSC_GKR ? 4 : P->ntab;
    if (table < 0 || table >= nt) return fail(EFFSC_INVALID_ARG, "table index out of range");
    *out = P->t[table].len;
    return EFFSC_OK;
}

int effsc_prover_read_table(effsc_prover* P, int table, uint64_t* out) {
    size_t n = 0;
    TRY(effsc_prover_table_len(P, table, &n));
    if (!n) return EFFSC_OK;
    if (!out) return fail(EFFSC_INVALID_ARG, "out is NULL");
    CK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = P->ctx->stream;
    Table& T = P->t[table];
    const Buf& b = T.bufs[T.cur];
    u64* stage = nullptr;
    CK(cudaMallocAsync((void**)&stage, n * (size_t)P->field * sizeof(u64), s));
    launch_join_aos(b.p[0], T.ext ? b.p[1] : nullptr, T.ext ? b.p[2] : nullptr, n, P->field, stage,
                    P->repr == EFFSC_MONTGOMERY, s);
    g_launches++;
    CK(cudaMemcpyAsync(out, stage, n * (size_t)P->field * sizeof(u64), cudaMemcpyDeviceToHost, s));
    CK(cudaFreeAsync(stage, s));
    CK(cudaStreamSynchronize(s));
    return EFFSC_OK;
}

int effsc_diag_bounded_wait(effsc_ctx* ctx, uint64_t limit_ns, int arrive, uint32_t* status_out) {
    if (!ctx || !status_out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    if (limit_ns > 2000000000ULL) return fail(EFFSC_INVALID_ARG, "limit above 2 s");
    CK(cudaSetDevice(ctx->device));
    u32* h = nullptr;
    u32* d = nullptr;
    CK(cudaHostAlloc((void**)&h, sizeof(u32), cudaHostAllocMapped));
    *h = 0xFFFFFFFFu;
    cudaError_t e = cudaHostGetDevicePointer((void**)&d, h, 0);
    if (e == cudaSuccess) {
        launch_diag_bounded_wait(limit_ns, arrive, d, ctx->stream);
        g_launches++;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    const u32 v = *(volatile u32*)h;
    cudaFreeHost(h);
    if (e != cudaSuccess) return fail(EFFSC_CUDA_ERROR, "bounded-wait self-test: %s", cudaGetErrorString(e));
    *status_out = v;
    return EFFSC_OK;
}

int effsc_prover_set_first_rounds(effsc_prover* P, int fused) {
    if (!P) return fail(EFFSC_INVALID_ARG, "prover is NULL");
    const int level = fused < 0 ? 0 : fused > 2 ? 2 : fused;
    if (level != P->fuse_first && P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    P->fuse_first = level;
    return EFFSC_OK;
}

int effsc_prover_set_persistent(effsc_prover* P, size_t max_len) {
    if (!P) return fail(EFFSC_INVALID_ARG, "prover is NULL");
    if (max_len != P->persist_len && P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    P->persist_len = max_len;
    return EFFSC_OK;
}

int effsc_prover_set_tail(effsc_prover* P, size_t max_len) {
    if (!P) return fail(EFFSC_INVALID_ARG, "prover is NULL");
    if (max_len != P->tail_len && P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    P->tail_len = max_len;
    return EFFSC_OK;
}

int effsc_prover_reset(effsc_prover* P) {
    if (!P) return fail(EFFSC_INVALID_ARG, "prover is NULL");
    for (int i = 0; i < 4; i++) {
        if (P->t[i].bufs.empty()) continue;
        P->t[i].cur = 0;
        P->t[i].len = P->len0[i];
        P->t[i].ext = P->ext0[i];
    }
    P->rounds = 0;
    return EFFSC_OK;
}

int effsc_prove(effsc_prover* P, size_t num_rounds, effsc_transcript* T, const uint8_t* hook, size_t hook_len,
                int use_graph, uint64_t* round_polys, uint64_t* challenges, uint64_t* final_value_out) {
    if (!P || !T) return fail(EFFSC_INVALID_ARG, "NULL argument");
    if (T->kind != EFFSC_T_KECCAK) return fail(EFFSC_UNSUPPORTED, "the device path needs a Keccak transcript");
    if (T->field != P->field) return fail(EFFSC_INVALID_ARG, "transcript field differs from the prover field");
    if (hook_len && !hook) return fail(EFFSC_INVALID_ARG, "hook is NULL");
    CK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = P->ctx->stream;
    const int d = degree_of(P);
    // device buffers for the proof and the transcript
    if (!P->d_tx) CK(cudaMallocAsync((void**)&P->d_tx, sizeof(DevTranscript), s));
    if (hook_len > P->hook_cap) {
        if (P->d_hook) CK(cudaFreeAsync(P->d_hook, s));
        CK(cudaMallocAsync((void**)&P->d_hook, hook_len, s));
        P->hook_cap = hook_len;
        if (P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    }
    if (num_rounds > P->rounds_cap || !P->d_wire) {
        if (P->d_wire) CK(cudaFreeAsync(P->d_wire, s));
        if (P->d_chals) CK(cudaFreeAsync(P->d_chals, s));
        size_t cap = std::max<size_t>(num_rounds, 1);
        CK(cudaMallocAsync((void**)&P->d_wire, cap * 9 * sizeof(u64), s));
        CK(cudaMallocAsync((void**)&P->d_chals, cap * 3 * sizeof(u64), s));
        if (P->h_out) { CK(cudaStreamSynchronize(s)); pinned_put(P->ctx, P->h_out, P->h_out_bytes); P->h_out = nullptr; }
        // sized in steps of 64 rounds so that provers of similar size share blocks
        const size_t capr = (cap + 63) / 64 * 64;
        P->h_out_bytes = (capr * 12 + TX_OUT_WORDS + 12) * sizeof(u64);
        P->h_out = (u64*)pinned_get(P->ctx, P->h_out_bytes);
        if (!P->h_out) return fail(EFFSC_OOM, "pinned output block");
        if (!P->d_first) CK(cudaMallocAsync((void**)&P->d_first, 12 * sizeof(u64), s));
        P->rounds_cap = cap;
        if (P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    }
    CK(cudaMemcpyAsync(P->d_tx, &T->st, sizeof(DevTranscript), cudaMemcpyHostToDevice, s));
    if (hook_len) CK(cudaMemcpyAsync(P->d_hook, hook, hook_len, cudaMemcpyHostToDevice, s));

    bool at_reset = P->rounds == 0;
    for (int i = 0; i < 4; i++)
        if (!P->t[i].bufs.empty() && (P->t[i].cur != 0 || P->t[i].len != P->len0[i])) at_reset = false;

    auto launch_all = [&](bool dry) -> int {
        size_t r0 = 0;
        bool tail_done = false;
        if (fuse3_ok(P, num_rounds)) {
            TxIO t0, t3;
            memset(&t0, 0, sizeof t0);
            t0.tx = P->d_tx;
            t0.hook = P->d_hook;
            t0.hook_len = (u32)hook_len;
            t3 = t0;
            t0.proof_wire = P->d_wire;
            t0.proof_chal = P->d_chals;
            t3.proof_wire = P->d_wire + (size_t)3 * 3 * d;
            t3.proof_chal = P->d_chals + 3 * 3;
            TRY(do_fuse3(P, t0, t3, P->d_chals, dry));
            r0 = 4;
        } else if (coef3_first_ok(P, num_rounds)) {
            TxIO t0, t2;
            memset(&t0, 0, sizeof t0);
            t0.tx = P->d_tx;
            t0.hook = P->d_hook;
            t0.hook_len = (u32)hook_len;
            t2 = t0;
            t0.proof_wire = P->d_wire;
            t0.proof_chal = P->d_chals;
            t2.proof_wire = P->d_wire + (size_t)2 * 3 * d;
            t2.proof_chal = P->d_chals + 3 * 2;
            TRY(do_coef3_first(P, t0, t2, P->d_chals, dry));
            r0 = 3;
        } else if (fuse_first_ok(P, num_rounds)) {
            TxIO t0, t2;
            memset(&t0, 0, sizeof t0);
            t0.tx = P->d_tx;
            t0.hook = P->d_hook;
            t0.hook_len = (u32)hook_len;
            t2 = t0;
            t0.proof_wire = P->d_wire;
            t0.proof_chal = P->d_chals;
            t2.proof_wire = P->d_wire + (size_t)2 * 3 * d;
            t2.proof_chal = P->d_chals + 3 * 2;
            TRY(do_fuse_first(P, t0, t2, P->d_chals, dry));
            r0 = 3;
        } else if (ml_first_ok(P, num_rounds)) {
            TxIO t0, t2;
            memset(&t0, 0, sizeof t0);
            t0.tx = P->d_tx;
            t0.hook = P->d_hook;
            t0.hook_len = (u32)hook_len;
            t2 = t0;
            t0.proof_wire = P->d_wire;
            t0.proof_chal = P->d_chals;
            t2.proof_wire = P->d_wire + (size_t)2 * 3 * d;
            t2.proof_chal = P->d_chals + 3 * 2;
            TRY(do_ml_first(P, t0, t2, P->d_chals, dry));
            r0 = 3;
        } else if (gkr_first_ok(P, num_rounds)) {
            TxIO t0, t2;
            memset(&t0, 0, sizeof t0);
            t0.tx = P->d_tx;
            t0.hook = P->d_hook;
            t0.hook_len = (u32)hook_len;
            t2 = t0;
            t0.proof_wire = P->d_wire;
            t0.proof_chal = P->d_chals;
            t2.proof_wire = P->d_wire + (size_t)2 * 3 * d;
            t2.proof_chal = P->d_chals + 3 * 2;
            TRY(do_gkr_first(P, t0, t2, P->d_chals, dry));
            r0 = 3;
        } else if (eqf_fast_ok(P, num_rounds)) {
            TxIO t0;
            memset(&t0, 0, sizeof t0);
            t0.tx = P->d_tx;
            t0.hook = P->d_hook;
            t0.hook_len = (u32)hook_len;
            t0.proof_wire = P->d_wire;
            t0.proof_chal = P->d_chals;
            TRY(do_eqf_left(P, t0, dry));
            r0 = P->v_l;
        }
        for (size_t r = r0; r < num_rounds; r++) {
            Chal ch;
            if (r > 0) { ch.has = true; ch.ext = P->field == EFFSC_FP3; ch.dev = P->d_chals + 3 * (r - 1); }
            TxIO tx;
            tx.tx = P->d_tx;
            tx.hook = P->d_hook;
            tx.hook_len = (u32)hook_len;
            tx.proof_wire = P->d_wire + (size_t)r * 3 * d;
            tx.proof_chal = P->d_chals + 3 * r;
            tx.chal_next = nullptr;
            // the tail runs the remaining rounds, the runner's finalize and
            // the read-back gather in its one launch
            if (tail_ok(P, r, num_rounds, ch)) {
                TRY(do_tail(P, r, num_rounds, ch, tx, dry, 0, true, P->d_first));
                tail_done = true;
                break;
            }
            if (gkr_tail_ok(P, r, num_rounds, ch)) {
                TRY(do_gkr_tail(P, r, num_rounds, ch, tx, dry, P->d_first));
                tail_done = true;
                break;
            }
            size_t nr = 0;
            if (persist_ok(P, r, num_rounds, ch, &nr)) {
                TRY(do_persist(P, r, nr, ch, hook_len, dry));
                r += nr - 1;
                continue;
            }
            u32 cs_log = 0;
            if (cluster_tail_ok(P, r, num_rounds, ch, &cs_log)) {
                TRY(do_tail(P, r, num_rounds, ch, tx, dry, cs_log, true, P->d_first));
                tail_done = true;
                break;
            }
            TRY(do_round(P, ch, tx, dry));
        }
        if (tail_done) return EFFSC_OK;
        if (num_rounds) {
            Chal ch;
            ch.has = true; ch.ext = P->field == EFFSC_FP3; ch.dev = P->d_chals + 3 * (num_rounds - 1);
            TRY(do_finalize(P, ch, dry));
        }
        if (!dry) {
            FirstSrc src;
            memset(&src, 0, sizeof src);
            for (int i = 0; i < 4; i++) {
                if (P->t[i].bufs.empty()) continue;
                const Buf& b = P->t[i].bufs[P->t[i].cur];
                for (int c = 0; c < (P->t[i].ext ? 3 : 1); c++) src.p[i][c] = b.p[c];
            }
            launch_gather_first(src, P->d_first, s);
            g_launches++;
        }
        return EFFSC_OK;
    };

    if (use_graph && at_reset && P->gexec && P->g_rounds == num_rounds && P->g_hook == hook_len) {
        CK(cudaGraphLaunch(P->gexec, s));
        g_launches += P->g_kernels;
        for (int i = 0; i < 4; i++) { P->t[i].cur = P->g_post[i].cur; P->t[i].len = P->g_post[i].len; P->t[i].ext = P->g_post[i].ext; }
        P->rounds = P->g_post_rounds;
    } else if (use_graph) {
        // plan once without launching so that every buffer exists before capture
        TabState pre[4];
        for (int i = 0; i < 4; i++) pre[i] = {P->t[i].cur, P->t[i].len, P->t[i].ext};
        size_t pre_rounds = P->rounds;
        TRY(launch_all(true));
        for (int i = 0; i < 4; i++) { P->t[i].cur = pre[i].cur; P->t[i].len = pre[i].len; P->t[i].ext = pre[i].ext; }
        P->rounds = pre_rounds;
        CK(cudaStreamSynchronize(s));
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        uint64_t before = g_launches;
        g_capturing = true;
        int rc = launch_all(false);
        g_capturing = false;
        cudaError_t ec = cudaStreamEndCapture(s, &graph);
        if (rc != EFFSC_OK) return rc;
        if (ec != cudaSuccess) return fail(EFFSC_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(ec));
        cudaGraphExec_t ge;
        ec = cudaGraphInstantiate(&ge, graph, 0);
        cudaGraphDestroy(graph);
        if (ec != cudaSuccess) return fail(EFFSC_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(ec));
        CK(cudaGraphLaunch(ge, s));
        if (at_reset) {
            P->g_kernels = g_launches - before;
            if (P->gexec) cudaGraphExecDestroy(P->gexec);
            P->gexec = ge;
            P->g_rounds = num_rounds;
            P->g_hook = hook_len;
            for (int i = 0; i < 4; i++) P->g_post[i] = {P->t[i].cur, P->t[i].len, P->t[i].ext};
            P->g_post_rounds = P->rounds;
        } else {
            CK(cudaStreamSynchronize(s));
            cudaGraphExecDestroy(ge);
        }
    } else {
        TRY(launch_all(false));
    }
    // results: pinned copies of the wire values, challenges, transcript state
    // and the tables' first entries, one synchronisation
    u64* hw = P->h_out;
    u64* hc = hw + num_rounds * 3 * d;
    u64* ht = hc + num_rounds * 3;
    u64* hf_ = ht + TX_OUT_WORDS;
    if (num_rounds) {
        CK(cudaMemcpyAsync(hw, P->d_wire, num_rounds * 3 * d * sizeof(u64), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hc, P->d_chals, num_rounds * 3 * sizeof(u64), cudaMemcpyDeviceToHost, s));
    }
    CK(cudaMemcpyAsync(ht, P->d_tx, sizeof(DevTranscript), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hf_, P->d_first, 12 * sizeof(u64), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    TRY(check_status(P));
    memcpy(&T->st, ht, sizeof(DevTranscript));
    for (size_t r = 0; r < num_rounds; r++) {
        if (round_polys)
            for (int i = 0; i < d; i++) {
                const u64* q = &hw[(r * d + i) * 3];
                store_elem(round_polys + (r * d + i) * P->field, hf(q[0], q[1], q[2]), P->field, P->repr);
            }
        if (challenges) store_elem(challenges + r * P->field, hf(hc[3 * r], hc[3 * r + 1], hc[3 * r + 2]), P->field, P->repr);
    }
    if (final_value_out) {
        HF v;
        g_first = hf_;
        int rc = final_value(P, &v);
        g_first = nullptr;
        TRY(rc);
        store_elem(final_value_out, v, P->field, P->repr);
    }
    return EFFSC_OK;
}

// ---- transcripts -----------------------------------------------------------
int effsc_transcript_create(int kind, int field, int repr, const uint8_t* label, size_t label_len, uint64_t seed,
                            effsc_transcript** out) {
    if (!out) return fail(EFFSC_INVALID_ARG, "out is NULL");
    TRY(check_field(field));
    if (kind != EFFSC_T_KECCAK && kind != EFFSC_T_TEST) return fail(EFFSC_INVALID_ARG, "unknown transcript kind");
    if (label_len && !label) return fail(EFFSC_INVALID_ARG, "label is NULL");
    effsc_transcript* t = new effsc_transcript();
    memset(&t->st, 0, sizeof t->st);
    t->kind = kind;
    t->field = field;
    t->repr = repr;
    t->st.deg = (u32)field;
    t->sm = seed;
    if (kind == EFFSC_T_KECCAK) {
        uint8_t l8[8];
        for (int i = 0; i < 8; i++) l8[i] = (uint8_t)((uint64_t)label_len >> (8 * i));
        tx_h_absorb(t, l8, 8);
        tx_h_absorb(t, label, label_len);
    }
    *out = t;
    return EFFSC_OK;
}
int effsc_transcript_destroy(effsc_transcript* t) { delete t; return EFFSC_OK; }
int effsc_transcript_clone(const effsc_transcript* t, effsc_transcript** out) {
    if (!t || !out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    *out = new effsc_transcript(*t);
    return EFFSC_OK;
}
int effsc_transcript_absorb(effsc_transcript* t, const uint8_t* b, size_t n) {
    if (!t || (n && !b)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    tx_h_absorb(t, b, n);
    return EFFSC_OK;
}
int effsc_transcript_squeeze(effsc_transcript* t, uint8_t* out, size_t n) {
    if (!t || (n && !out)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    if (t->kind != EFFSC_T_KECCAK) return fail(EFFSC_UNSUPPORTED, "squeeze needs a Keccak transcript");
    tx_h_squeeze(t, out, n);
    return EFFSC_OK;
}
int effsc_transcript_send(effsc_transcript* t, const uint64_t* v) {
    if (!t || !v) return fail(EFFSC_INVALID_ARG, "NULL argument");
    tx_h_send(t, load_elem(v, t->field, t->repr));
    return EFFSC_OK;
}
int effsc_transcript_challenge(effsc_transcript* t, uint64_t* out) {
    if (!t || !out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    store_elem(out, tx_h_challenge(t), t->field, t->repr);
    return EFFSC_OK;
}

// ---- verifier (src/verifier.rs:61-184) -------------------------------------
int effsc_verify(int field, int repr, const uint64_t* claimed_sum, size_t degree, size_t num_rounds,
                 effsc_transcript* t, const uint8_t* hook, size_t hook_len, const uint64_t* round_polys,
                 uint64_t* challenges, uint64_t* final_claim) {
    if (!t || !claimed_sum || (num_rounds && !round_polys) || !final_claim) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (degree > 8) return fail(EFFSC_INVALID_ARG, "degree too large");
    HF claim = load_elem(claimed_sum, field, repr);
    const size_t dd = degree, n_wire = dd > 1 ? dd : 1;
    for (size_t round = 0; round < num_rounds; round++) {
        HF recv[8];
        for (size_t i = 0; i < n_wire; i++) {
            recv[i] = load_elem(round_polys + (round * n_wire + i) * (size_t)field, field, repr);
            tx_h_send(t, recv[i]);
        }
        HF h0 = recv[0], h1 = hf_sub(claim, h0);
        if (hook_len) tx_h_absorb(t, hook, hook_len);
        HF r = tx_h_challenge(t);
        if (challenges) store_elem(challenges + round * (size_t)field, r, field, repr);
        if (dd == 0) { claim = h0; continue; }
        HF hinf = dd >= 2 ? recv[1] : hf_sub(h1, h0);
        HF q[8];
        q[0] = h0;
        q[1] = hf_sub(h1, hinf);
        for (size_t i = 2; i < dd; i++) {
            HF id = hf(1), fi = hf_from_u64(i);
            for (size_t k = 0; k < dd; k++) id = hf_mul(id, fi);
            q[i] = hf_sub(recv[i], hf_mul(hinf, id));
        }
        HF qr;
        if (dd == 1) qr = q[0];
        else if (dd == 2) qr = hf_add(q[0], hf_mul(r, hf_sub(q[1], q[0])));
        else {
            // Lagrange at {0..dd-1} with barycentric weights prod_{j != i} (i - j)
            HF pre[9], suf[9], rm[8];
            for (size_t j = 0; j < dd; j++) rm[j] = hf_sub(r, hf_from_u64(j));
            pre[0] = hf(1);
            for (size_t i = 0; i < dd; i++) pre[i + 1] = hf_mul(pre[i], rm[i]);
            suf[dd] = hf(1);
            for (size_t i = dd; i-- > 0;) suf[i] = hf_mul(suf[i + 1], rm[i]);
            qr = hf(0);
            for (size_t i = 0; i < dd; i++) {
                u64 w = 1;
                for (size_t j = 0; j < dd; j++) {
                    if (j == i) continue;
                    long long diff = (long long)i - (long long)j;
                    w = h_mul(w, diff > 0 ? (u64)diff : h_sub(0, (u64)(-diff)));
                }
                qr = hf_add(qr, hf_mul(hf_mul(q[i], hf_mul(pre[i], suf[i + 1])), hf(h_inv(w))));
            }
        }
        HF rd = hf(1);
        for (size_t k = 0; k < dd; k++) rd = hf_mul(rd, r);
        claim = hf_add(qr, hf_mul(hinf, rd));
    }
    store_elem(final_claim, claim, field, repr);
    return EFFSC_OK;
}

// ---- standalone fold, eq table, generator ------------------------------------
int effsc_fold(effsc_ctx* ctx, int field, int repr, const uint64_t* values, size_t len, int ncomp,
               const uint64_t* weight, uint64_t* out, size_t* out_len) {
    if (!ctx || !weight || !out_len || (len && (!values || !out))) return fail(EFFSC_INVALID_ARG, "NULL argument");
    const uint64_t* tabs[1] = {values};
    size_t lens[1] = {len};
    int nc[1] = {ncomp};
    effsc_prover* P = nullptr;
    TRY(effsc_prover_create(ctx, EFFSC_ML, EFFSC_MSB, field, repr, 1, tabs, lens, nc, &P));
    int rc = do_finalize(P, host_chal(P, weight), false);
    if (rc == EFFSC_OK) {
        *out_len = P->t[0].len;
        rc = effsc_prover_read_table(P, 0, out);
    }
    release_prover(P);
    return rc;
}

int effsc_compute_sumcheck_polynomial(effsc_ctx* ctx, int field, int repr, const uint64_t* values, size_t len,
                                      int ncomp, uint64_t* out_s0_s1) {
    if (!ctx || !out_s0_s1 || (len && !values)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (!len) {
        // src/multilinear_sumcheck.rs:110-112: an empty table gives (0, 0)
        memset(out_s0_s1, 0, 2 * (size_t)field * sizeof(uint64_t));
        return EFFSC_OK;
    }
    const uint64_t* tabs[1] = {values};
    size_t lens[1] = {len};
    int nc[1] = {ncomp};
    effsc_prover* P = nullptr;
    TRY(effsc_prover_create(ctx, EFFSC_ML, EFFSC_MSB, field, repr, 1, tabs, lens, nc, &P));
    int rc = effsc_prover_round(P, nullptr, nullptr, out_s0_s1);
    release_prover(P);
    return rc;
}

int effsc_fused_fold_and_compute_polynomial(effsc_ctx* ctx, int field, int repr, const uint64_t* values, size_t len,
                                            int ncomp, const uint64_t* weight, uint64_t* out, size_t* out_len,
                                            uint64_t* out_s0_s1) {
    if (!ctx || !weight || !out_len || !out_s0_s1 || (len && (!values || !out)))
        return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (!len) {
        *out_len = 0;
        memset(out_s0_s1, 0, 2 * (size_t)field * sizeof(uint64_t));
        return EFFSC_OK;
    }
    const uint64_t* tabs[1] = {values};
    size_t lens[1] = {len};
    int nc[1] = {ncomp};
    effsc_prover* P = nullptr;
    TRY(effsc_prover_create(ctx, EFFSC_ML, EFFSC_MSB, field, repr, 1, tabs, lens, nc, &P));
    // a round with a challenge: the fold (fused with the evaluation for
    // power-of-two lengths >= 4, else fold then evaluate) and the new (s0, s1)
    int rc = effsc_prover_round(P, weight, nullptr, out_s0_s1);
    if (rc == EFFSC_OK) {
        *out_len = P->t[0].len;
        rc = effsc_prover_read_table(P, 0, out);
    }
    release_prover(P);
    return rc;
}

int effsc_build_eq_table(effsc_ctx* ctx, int field, int repr, const uint64_t* w, size_t num_vars, uint64_t* out) {
    if (!ctx || !out || (num_vars && !w)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    TRY(check_field(field));
    if (num_vars > 34) return fail(EFFSC_INVALID_ARG, "num_vars too large");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    std::vector<u64> wc(3 * (num_vars ? num_vars : 1), 0);
    bool ext = false;
    for (size_t j = 0; j < num_vars; j++) {
        HF x = load_elem(w + j * (size_t)field, field, repr);
        for (int c = 0; c < 3; c++) wc[3 * j + c] = x.c[c];
        ext |= hf_is_ext(x);
    }
    size_t n = (size_t)1 << num_vars;
    u64 *dw = nullptr, *c0 = nullptr, *c1 = nullptr, *c2 = nullptr, *stage = nullptr;
    CK(cudaMallocAsync((void**)&dw, wc.size() * sizeof(u64), s));
    CK(cudaMemcpyAsync(dw, wc.data(), wc.size() * sizeof(u64), cudaMemcpyHostToDevice, s));
    CK(cudaMallocAsync((void**)&c0, n * sizeof(u64), s));
    if (ext) { CK(cudaMallocAsync((void**)&c1, n * sizeof(u64), s)); CK(cudaMallocAsync((void**)&c2, n * sizeof(u64), s)); }
    launch_build_eq(dw, (u32)num_vars, ext, c0, c1, c2, s);
    g_launches++;
    CK(cudaMallocAsync((void**)&stage, n * (size_t)field * sizeof(u64), s));
    launch_join_aos(c0, c1, c2, n, field, stage, repr == EFFSC_MONTGOMERY, s);
    g_launches++;
    CK(cudaMemcpyAsync(out, stage, n * (size_t)field * sizeof(u64), cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(dw, s); cudaFreeAsync(c0, s); if (c1) cudaFreeAsync(c1, s); if (c2) cudaFreeAsync(c2, s); cudaFreeAsync(stage, s);
    CK(cudaStreamSynchronize(s));
    return EFFSC_OK;
}

uint64_t effsc_table_seed(uint64_t seed, uint64_t table) {
    u64 z = seed + (table + 1) * 0x632BE59BD9B4E019ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

int effsc_gen_uniform(effsc_ctx* ctx, uint64_t seed, uint64_t n, uint64_t* dev_out, uint64_t* host_out) {
    if (!ctx || (!dev_out && !host_out)) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    u64* d = (u64*)dev_out;
    if (!d) CK(cudaMallocAsync((void**)&d, (n ? n : 1) * sizeof(u64), s));
    launch_gen_uniform(seed, n, d, s);
    g_launches++;
    if (host_out && n) CK(cudaMemcpyAsync(host_out, d, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
    if (!dev_out) CK(cudaFreeAsync(d, s));
    CK(cudaStreamSynchronize(s));
    return EFFSC_OK;
}

int effsc_device_alloc(effsc_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
    if (e != cudaSuccess) return fail(EFFSC_OOM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return EFFSC_OK;
}
int effsc_device_free(effsc_ctx* ctx, void* p) {
    if (!ctx) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaFree(p));
    return EFFSC_OK;
}
int effsc_memcpy_h2d(effsc_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!ctx) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return EFFSC_OK;
}
int effsc_memcpy_d2h(effsc_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (!ctx) return fail(EFFSC_INVALID_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return EFFSC_OK;
}

}  // extern "C"
