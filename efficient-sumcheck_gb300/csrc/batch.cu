// batch.cu -- many independent Multilinear / InnerProduct (MSB) provers of
// uneven size proved together: one kernel launch per step for every instance
// still in its multi-block rounds (k_serve_step: each instance's segment runs
// its own round, or the two-pass start of an InnerProduct proof over Fp3),
// one launch of the one-block tail kernel for every instance's last rounds,
// one launch for all final folds; each instance keeps its own grid reduction
// and Keccak transcript, and the whole protocol is captured once as a CUDA
// graph.
//
// Instance i has num_vars[i] = n_i variables (tables of 2^n_i elements) and is
// proved with all n_i rounds, exactly as runner::sumcheck (src/runner.rs:29-69)
// would prove it alone with a transcript labelled by the caller; its proof is
// bit-identical to the single-instance path (tests/test_batch.py).
#include "effsc_gpu.h"
#include "kernels.h"
#include "keccak.cuh"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace effsc;

void effsc_internal_tx_state(const effsc_transcript* t, void* out);
int effsc_internal_ctx_device(const effsc_ctx* c);
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c);

#define BCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

struct effsc_batch {
    effsc_ctx* ctx = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    int kind = EFFSC_IP, field = EFFSC_FP3, ntab = 2, pol = POL_IP;
    size_t n = 0;
    std::vector<u32> nv;
    std::vector<size_t> round_off;         // prefix sums of nv: proof row of instance i
    size_t total_rounds = 0;
    u32 max_nv = 0;
    // device memory: one pool
    u64* pool = nullptr;
    std::vector<u64*> in;                  // n * ntab base input tables
    std::vector<u64*> work;                // n * ntab work tables (3 component arrays for Fp3)
    // schedule
    int quads_per_thread = 2;
    u64 tail_len = ~0ULL;                  // tables of at most this length finish in the tail kernel
    bool planned = false;
    std::vector<u32> tail_r0;              // first tail round per instance (nv[i]: no tail)
    TailArgs* d_tail = nullptr;
    u32 n_tail = 0;
    u64 tail_smem_len = 0;
    u32 rounds_planned = 0;                // step launches before the tail
    std::vector<size_t> seg_off, seg_cnt;  // per step into d_segs / d_args
    std::vector<u32> grid;                 // blocks per step
    ServeSeg* d_segs = nullptr;
    RoundArgs* d_args = nullptr;           // one RoundArgs per segment, steps concatenated
    RoundArgs* d_fin_args = nullptr;
    unsigned char* d_ext = nullptr;
    u64* d_partials = nullptr;
    u32* d_counters = nullptr;
    u32* h_status = nullptr;
    u32* d_status = nullptr;
    DevTranscript* d_tx = nullptr;
    u64* d_wire = nullptr;
    u64* d_chal = nullptr;
    u64* d_final = nullptr;
    cudaGraphExec_t gexec = nullptr;
    uint64_t graph_kernels = 0;
    u64* h_out = nullptr;                  // pinned: wire rows | challenge rows | final values
};

namespace {

int deg_of(const effsc_batch* b) { return b->kind == EFFSC_ML ? 1 : 2; }

void free_schedule(effsc_batch* b) {
    cudaStream_t s = b->stream;
    if (b->d_segs) cudaFreeAsync(b->d_segs, s);
    if (b->d_args) cudaFreeAsync(b->d_args, s);
    if (b->d_fin_args) cudaFreeAsync(b->d_fin_args, s);
    if (b->d_ext) cudaFreeAsync(b->d_ext, s);
    if (b->d_partials) cudaFreeAsync(b->d_partials, s);
    if (b->d_tail) cudaFreeAsync(b->d_tail, s);
    b->d_tail = nullptr;
    b->n_tail = 0;
    b->d_segs = nullptr; b->d_args = nullptr; b->d_fin_args = nullptr; b->d_ext = nullptr; b->d_partials = nullptr;
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    b->planned = false;
}

// Build every round's segments and per-instance RoundArgs.
int plan(effsc_batch* b) {
    free_schedule(b);
    const int F3W = b->field == EFFSC_FP3 ? 3 : 1;
    // tail switch: instance i runs rounds tail_r0[i] .. n_i - 1 in the one-block
    // tail kernel, starting from a table of at most `tl` entries
    const u64 tl = std::min<u64>(b->tail_len, tail_max_len(b->pol, F3W, TAIL_SMEM_CAP));
    u32 tail_log = 0;
    while ((2ULL << tail_log) <= tl) tail_log++;
    b->tail_r0.assign(b->n, 0);
    for (size_t i = 0; i < b->n; i++) {
        const u32 n_i = b->nv[i];
        if (tail_log < 2) b->tail_r0[i] = n_i;
        else b->tail_r0[i] = n_i <= tail_log ? 0 : n_i - tail_log + 1;
    }
    // steps: one launch each.  An InnerProduct instance over Fp3 whose first
    // three rounds are all multi-block takes two steps for them (ip01.cuh:
    // rounds 0-1, then round 2 with the double fold); every other round is
    // one step.  Step s of instance i runs round s, or for the two-pass
    // start: rounds 0-1 (s = 0), round 2 (s = 1), round s + 1 (s >= 2).
    const int maxb = max_grid();
    std::vector<char> two(b->n, 0);
    std::vector<u32> nsteps(b->n, 0);
    u32 S = 0;
    for (size_t i = 0; i < b->n; i++) {
        two[i] = b->kind == EFFSC_IP && F3W == 3 && b->tail_r0[i] >= 3;
        nsteps[i] = two[i] ? b->tail_r0[i] - 1 : b->tail_r0[i];
        S = std::max<u32>(S, nsteps[i]);
    }
    std::vector<ServeSeg> segs;
    std::vector<RoundArgs> args;
    b->rounds_planned = S;
    b->seg_off.assign(S, 0);
    b->seg_cnt.assign(S, 0);
    b->grid.assign(S, 0);
    size_t max_blocks = 1;
    std::vector<RoundArgs> fin(b->n);
    std::vector<unsigned char> ext(b->n, 0);
    const u64 per_block = (u64)KERNEL_TPB * b->quads_per_thread;
    const u32 kind_code = (b->kind == EFFSC_IP ? SERVE_IP : 0) | (F3W == 3 ? SERVE_FP3 : 0);
    for (u32 st = 0; st < S; st++) {
        b->seg_off[st] = segs.size();
        u32 first = 0;
        for (size_t i = 0; i < b->n; i++) {
            if (st >= nsteps[i]) continue;
            const u32 n_i = b->nv[i];
            const u64 half0 = 1ULL << (n_i - 1);      // work buffer length (one component)
            RoundArgs a;
            memset(&a, 0, sizeof a);
            u32 phase, r;
            u64 L, work;
            if (two[i] && st < 2) {
                r = st == 0 ? 0 : 2;
                phase = st == 0 ? SERVE_IP01 : SERVE_IP2X;
                L = 1ULL << n_i;
                work = st == 0 ? L / 4 : L / 8;
                for (int t = 0; t < 2; t++) {
                    a.t[t].in[0] = b->in[i * 2 + t];
                    if (st) for (int c = 0; c < 3; c++) a.t[t].out[c] = b->work[i * 2 + t] + c * half0;
                }
                a.chal_ptr = st ? b->d_chal + 3 * b->round_off[i] : nullptr;
                a.chal2_ptr = st ? b->d_chal + 3 * (b->round_off[i] + 1) : nullptr;
            } else {
                r = two[i] ? st + 1 : st;
                L = r == 0 ? (1ULL << n_i) : (1ULL << (n_i - r + 1));
                work = r == 0 ? L / 2 : L / 4;
                phase = r == 0 ? SERVE_EVAL : (r == 1 || F3W == 1) ? SERVE_FOLD_BASE : SERVE_FOLD_EXT;
                for (int t = 0; t < b->ntab; t++) {
                    u64* inb = b->in[i * b->ntab + t];
                    u64* wk = b->work[i * b->ntab + t];
                    const bool cur_ext = r >= 2 && F3W == 3;
                    if (r <= 1) a.t[t].in[0] = inb;
                    else for (int c = 0; c < (cur_ext ? 3 : 1); c++) a.t[t].in[c] = wk + c * half0;
                    if (r >= 1)
                        for (int c = 0; c < F3W; c++) a.t[t].out[c] = wk + c * half0;
                }
                a.chal_ptr = r ? b->d_chal + 3 * (b->round_off[i] + r - 1) : nullptr;
            }
            u64 nb = (work + per_block - 1) / per_block;
            nb = std::max<u64>(1, std::min<u64>(nb, (u64)maxb));
            ServeSeg sg;
            sg.first_block = first;
            sg.nblocks = (u32)nb;
            sg.code = kind_code | (phase << SERVE_PHASE_SHIFT);
            sg.reserved = 0;
            segs.push_back(sg);
            a.L = L;
            a.counter = b->d_counters + i;
            a.status = b->d_status;
            a.tx.tx = b->d_tx + i;
            a.tx.proof_wire = b->d_wire + 3 * deg_of(b) * (b->round_off[i] + r);
            a.tx.proof_chal = b->d_chal + 3 * (b->round_off[i] + r);
            args.push_back(a);
            first += (u32)nb;
        }
        b->seg_cnt[st] = segs.size() - b->seg_off[st];
        b->grid[st] = first;
        max_blocks = std::max<size_t>(max_blocks, first);
    }
    // finalize: the tables after round n_i - 1 (length 2)
    for (size_t i = 0; i < b->n; i++) {
        const u32 n_i = b->nv[i];
        RoundArgs a;
        memset(&a, 0, sizeof a);
        const bool e = n_i >= 2 && F3W == 3;
        for (int t = 0; t < b->ntab; t++) {
            u64* inb = b->in[i * b->ntab + t];
            u64* wk = b->work[i * b->ntab + t];
            const u64 half0 = 1ULL << (n_i - 1);
            if (n_i == 1) a.t[t].in[0] = inb;
            else for (int c = 0; c < (e ? 3 : 1); c++) a.t[t].in[c] = wk + c * half0;
        }
        a.chal_ptr = b->d_chal + 3 * (b->round_off[i] + n_i - 1);
        fin[i] = a;
        ext[i] = e ? 1 : 0;
    }
    // tail kernel arguments (one block per instance with tail rounds)
    std::vector<TailArgs> tails;
    b->tail_smem_len = 0;
    for (size_t i = 0; i < b->n; i++) {
        const u32 n_i = b->nv[i], r0 = b->tail_r0[i];
        if (r0 >= n_i) continue;
        TailArgs ta;
        memset(&ta, 0, sizeof ta);
        ta.L = r0 == 0 ? (1ULL << n_i) : (1ULL << (n_i - r0 + 1));
        const u32 folds = n_i - r0 - (r0 == 0 ? 1 : 0);
        const u64 half0 = 1ULL << (n_i - 1);
        for (int t = 0; t < b->ntab; t++) {
            u64* inb = b->in[i * b->ntab + t];
            u64* wk = b->work[i * b->ntab + t];
            if (r0 <= 1) ta.in[t][0] = inb;
            else {
                for (int c = 0; c < F3W; c++) ta.in[t][c] = wk + c * half0;
                if (F3W == 3) ta.in_ext |= 1u << t;
            }
            if (folds)
                for (int c = 0; c < F3W; c++) ta.out[t][c] = wk + c * half0;
        }
        ta.nrounds = n_i - r0;
        ta.first_fold = r0 >= 1;
        ta.chal_in = r0 >= 1 ? b->d_chal + 3 * (b->round_off[i] + r0 - 1) : nullptr;
        ta.tx = b->d_tx + i;
        ta.proof_wire = b->d_wire + 3 * deg_of(b) * (b->round_off[i] + r0);
        ta.proof_chal = b->d_chal + 3 * (b->round_off[i] + r0);
        tails.push_back(ta);
        b->tail_smem_len = std::max<u64>(b->tail_smem_len, ta.L);
    }
    cudaStream_t s = b->stream;
    BCK(cudaMallocAsync((void**)&b->d_partials, max_blocks * 12 * sizeof(u64), s));
    b->n_tail = (u32)tails.size();
    if (!tails.empty()) {
        BCK(cudaMallocAsync((void**)&b->d_tail, tails.size() * sizeof(TailArgs), s));
        BCK(cudaMemcpyAsync(b->d_tail, tails.data(), tails.size() * sizeof(TailArgs), cudaMemcpyHostToDevice, s));
    }
    // per-segment partial ranges: block-index offsets within each step
    for (size_t k = 0; k < segs.size(); k++) args[k].partials = b->d_partials + (size_t)segs[k].first_block * 12;
    BCK(cudaMallocAsync((void**)&b->d_segs, std::max<size_t>(1, segs.size()) * sizeof(ServeSeg), s));
    BCK(cudaMallocAsync((void**)&b->d_args, std::max<size_t>(1, args.size()) * sizeof(RoundArgs), s));
    BCK(cudaMallocAsync((void**)&b->d_fin_args, std::max<size_t>(1, fin.size()) * sizeof(RoundArgs), s));
    BCK(cudaMallocAsync((void**)&b->d_ext, std::max<size_t>(1, ext.size()), s));
    if (!segs.empty()) BCK(cudaMemcpyAsync(b->d_segs, segs.data(), segs.size() * sizeof(ServeSeg), cudaMemcpyHostToDevice, s));
    if (!args.empty()) BCK(cudaMemcpyAsync(b->d_args, args.data(), args.size() * sizeof(RoundArgs), cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(b->d_fin_args, fin.data(), fin.size() * sizeof(RoundArgs), cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(b->d_ext, ext.data(), ext.size(), cudaMemcpyHostToDevice, s));
    BCK(cudaStreamSynchronize(s));
    b->planned = true;
    return EFFSC_OK;
}

int launch_protocol(effsc_batch* b, uint64_t* kernels) {
    for (u32 st = 0; st < b->rounds_planned; st++) {
        if (!b->seg_cnt[st]) continue;
        launch_serve_step(b->d_segs + b->seg_off[st], (u32)b->seg_cnt[st], b->d_args + b->seg_off[st], b->grid[st],
                          b->stream);
        (*kernels)++;
    }
    if (b->n_tail) {
        if (!launch_tail(b->pol, b->field == EFFSC_FP3 ? 3 : 1, b->d_tail, nullptr, b->n_tail, b->tail_smem_len, b->stream))
            return effsc_set_error(EFFSC_UNSUPPORTED, "no tail kernel for this batch");
        (*kernels)++;
    }
    launch_batch_finalize(b->d_fin_args, b->d_ext, (u32)b->n, b->ntab, b->d_final, b->stream);
    (*kernels)++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "batched round launch: %s", cudaGetErrorString(e));
    return EFFSC_OK;
}

}  // namespace

uint64_t effsc_internal_add_launches(uint64_t k);

extern "C" {

int effsc_batch_create(effsc_ctx* ctx, int kind, int field, size_t n_inst, const uint32_t* num_vars,
                       const uint64_t* const* host_tables, const uint64_t* seeds, effsc_batch** out) {
    if (!ctx || !out || !num_vars || (!host_tables && !seeds) || !n_inst)
        return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument or empty batch");
    if (kind != EFFSC_IP && kind != EFFSC_ML) return effsc_set_error(EFFSC_UNSUPPORTED, "batches hold IP or ML provers");
    if (field != EFFSC_FP && field != EFFSC_FP3) return effsc_set_error(EFFSC_INVALID_ARG, "bad field");
    for (size_t i = 0; i < n_inst; i++)
        if (num_vars[i] < 1 || num_vars[i] > 34) return effsc_set_error(EFFSC_INVALID_ARG, "num_vars[%zu] = %u out of range 1..34", i, num_vars[i]);
    BCK(cudaSetDevice(effsc_internal_ctx_device(ctx)));
    effsc_batch* b = new effsc_batch();
    b->ctx = ctx;
    b->device = effsc_internal_ctx_device(ctx);
    b->stream = effsc_internal_ctx_stream(ctx);
    b->kind = kind;
    b->field = field;
    b->ntab = kind == EFFSC_IP ? 2 : 1;
    b->pol = kind == EFFSC_IP ? POL_IP : POL_ML;
    b->n = n_inst;
    b->nv.assign(num_vars, num_vars + n_inst);
    b->round_off.resize(n_inst + 1);
    b->round_off[0] = 0;
    for (size_t i = 0; i < n_inst; i++) {
        b->round_off[i + 1] = b->round_off[i] + b->nv[i];
        b->max_nv = std::max<u32>(b->max_nv, b->nv[i]);
    }
    b->total_rounds = b->round_off[n_inst];
    const int F3W = field == EFFSC_FP3 ? 3 : 1;
    // one pool: inputs (2^n words per table) then work buffers (F3W * 2^(n-1))
    size_t words = 0;
    for (size_t i = 0; i < n_inst; i++) words += (size_t)b->ntab * ((1ULL << b->nv[i]) + F3W * (1ULL << (b->nv[i] - 1)));
    cudaStream_t s = b->stream;
    auto bail = [&](int rc) { effsc_batch_destroy(b); return rc; };
    cudaError_t e = cudaMallocAsync((void**)&b->pool, words * sizeof(u64), s);
    if (e != cudaSuccess) { delete b; return effsc_set_error(EFFSC_OOM, "batch pool of %zu bytes: %s", words * 8, cudaGetErrorString(e)); }
    size_t off = 0;
    b->in.resize(n_inst * b->ntab);
    b->work.resize(n_inst * b->ntab);
    for (size_t i = 0; i < n_inst; i++)
        for (int t = 0; t < b->ntab; t++) {
            const size_t L = 1ULL << b->nv[i];
            b->in[i * b->ntab + t] = b->pool + off;
            off += L;
            b->work[i * b->ntab + t] = b->pool + off;
            off += F3W * (L / 2);
        }
    for (size_t i = 0; i < n_inst; i++)
        for (int t = 0; t < b->ntab; t++) {
            const size_t L = 1ULL << b->nv[i];
            u64* dst = b->in[i * b->ntab + t];
            if (host_tables) {
                if (!host_tables[i * b->ntab + t]) return bail(effsc_set_error(EFFSC_INVALID_ARG, "table %zu/%d is NULL", i, t));
                e = cudaMemcpyAsync(dst, host_tables[i * b->ntab + t], L * sizeof(u64), cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess) return bail(effsc_set_error(EFFSC_CUDA_ERROR, "upload: %s", cudaGetErrorString(e)));
            } else {
                launch_gen_uniform(seeds[i * b->ntab + t], L, dst, s);
            }
        }
    if (cudaMallocAsync((void**)&b->d_counters, n_inst * sizeof(u32), s) != cudaSuccess ||
        cudaMemsetAsync(b->d_counters, 0, n_inst * sizeof(u32), s) != cudaSuccess ||
        cudaMallocAsync((void**)&b->d_tx, n_inst * sizeof(DevTranscript), s) != cudaSuccess ||
        cudaMallocAsync((void**)&b->d_wire, std::max<size_t>(1, b->total_rounds) * 3 * 2 * sizeof(u64), s) != cudaSuccess ||
        cudaMallocAsync((void**)&b->d_chal, std::max<size_t>(1, b->total_rounds) * 3 * sizeof(u64), s) != cudaSuccess ||
        cudaMallocAsync((void**)&b->d_final, n_inst * 3 * sizeof(u64), s) != cudaSuccess)
        return bail(effsc_set_error(EFFSC_OOM, "batch bookkeeping allocation failed"));
    const size_t rows = std::max<size_t>(1, b->total_rounds);
    if (cudaHostAlloc((void**)&b->h_out, (rows * 3 * 2 + rows * 3 + n_inst * 3) * sizeof(u64), cudaHostAllocDefault) != cudaSuccess)
        return bail(effsc_set_error(EFFSC_OOM, "pinned output staging"));
    if (cudaHostAlloc((void**)&b->h_status, sizeof(u32), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&b->d_status, b->h_status, 0) != cudaSuccess)
        return bail(effsc_set_error(EFFSC_CUDA_ERROR, "mapped status word"));
    *b->h_status = 0;
    int rc = plan(b);
    if (rc != EFFSC_OK) return bail(rc);
    *out = b;
    return EFFSC_OK;
}

int effsc_batch_destroy(effsc_batch* b) {
    if (!b) return EFFSC_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    free_schedule(b);
    cudaStream_t s = b->stream;
    if (b->pool) cudaFreeAsync(b->pool, s);
    if (b->d_counters) cudaFreeAsync(b->d_counters, s);
    if (b->d_tx) cudaFreeAsync(b->d_tx, s);
    if (b->d_wire) cudaFreeAsync(b->d_wire, s);
    if (b->d_chal) cudaFreeAsync(b->d_chal, s);
    if (b->d_final) cudaFreeAsync(b->d_final, s);
    cudaStreamSynchronize(s);
    if (b->h_status) cudaFreeHost(b->h_status);
    if (b->h_out) cudaFreeHost(b->h_out);
    delete b;
    return EFFSC_OK;
}

int effsc_batch_set_quads_per_thread(effsc_batch* b, int q) {
    if (!b || q < 1 || q > 64) return effsc_set_error(EFFSC_INVALID_ARG, "quads_per_thread must be 1..64");
    if (q == b->quads_per_thread && b->planned) return EFFSC_OK;
    BCK(cudaSetDevice(b->device));
    b->quads_per_thread = q;
    return plan(b);
}

int effsc_batch_set_tail(effsc_batch* b, uint64_t max_len) {
    if (!b) return effsc_set_error(EFFSC_INVALID_ARG, "NULL batch");
    if (max_len == b->tail_len && b->planned) return EFFSC_OK;
    BCK(cudaSetDevice(b->device));
    b->tail_len = max_len;
    return plan(b);
}

int effsc_batch_device_table(effsc_batch* b, size_t inst, int table, const uint64_t** out) {
    if (!b || !out || inst >= b->n || table < 0 || table >= b->ntab) return effsc_set_error(EFFSC_INVALID_ARG, "bad index");
    *out = (const uint64_t*)b->in[inst * b->ntab + table];
    return EFFSC_OK;
}

int effsc_batch_prove(effsc_batch* b, const effsc_transcript* const* transcripts, int use_graph,
                      uint64_t* round_polys, uint64_t* challenges, uint64_t* final_values) {
    if (!b || !transcripts) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    BCK(cudaSetDevice(b->device));
    cudaStream_t s = b->stream;
    std::vector<DevTranscript> st(b->n);
    for (size_t i = 0; i < b->n; i++) {
        if (!transcripts[i]) return effsc_set_error(EFFSC_INVALID_ARG, "transcript %zu is NULL", i);
        effsc_internal_tx_state(transcripts[i], &st[i]);
        if ((int)st[i].deg != b->field) return effsc_set_error(EFFSC_INVALID_ARG, "transcript %zu: wrong field or kind", i);
    }
    BCK(cudaMemcpyAsync(b->d_tx, st.data(), st.size() * sizeof(DevTranscript), cudaMemcpyHostToDevice, s));
    uint64_t kernels = 0;
    if (use_graph) {
        if (!b->gexec) {
            BCK(cudaStreamSynchronize(s));
            cudaGraph_t g;
            BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int rc = launch_protocol(b, &kernels);
            cudaError_t ec = cudaStreamEndCapture(s, &g);
            if (rc != EFFSC_OK) return rc;
            if (ec != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "batch graph capture: %s", cudaGetErrorString(ec));
            ec = cudaGraphInstantiate(&b->gexec, g, 0);
            cudaGraphDestroy(g);
            if (ec != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "batch graph instantiate: %s", cudaGetErrorString(ec));
            b->graph_kernels = kernels;
        }
        BCK(cudaGraphLaunch(b->gexec, s));
        kernels = b->graph_kernels;
    } else {
        int rc = launch_protocol(b, &kernels);
        if (rc != EFFSC_OK) return rc;
    }
    effsc_internal_add_launches(kernels);
    const int d = deg_of(b), f = b->field;
    u64* wire = b->h_out;
    u64* chal = wire + b->total_rounds * 3 * d;
    u64* fin = chal + b->total_rounds * 3;
    if (round_polys) BCK(cudaMemcpyAsync(wire, b->d_wire, b->total_rounds * 3 * d * 8, cudaMemcpyDeviceToHost, s));
    if (challenges) BCK(cudaMemcpyAsync(chal, b->d_chal, b->total_rounds * 3 * 8, cudaMemcpyDeviceToHost, s));
    if (final_values) BCK(cudaMemcpyAsync(fin, b->d_final, b->n * 3 * 8, cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    if (*(volatile u32*)b->h_status) {
        *(volatile u32*)b->h_status = 0;
        cudaMemsetAsync(b->d_counters, 0, b->n * sizeof(u32), s);
        return effsc_set_error(EFFSC_TIMEOUT, "a batched round kernel timed out");
    }
    for (size_t row = 0; row < b->total_rounds; row++) {
        if (round_polys)
            for (int k = 0; k < d; k++)
                for (int c = 0; c < f; c++) round_polys[(row * d + k) * f + c] = wire[(row * d + k) * 3 + c];
        if (challenges)
            for (int c = 0; c < f; c++) challenges[row * f + c] = chal[row * 3 + c];
    }
    if (final_values)
        for (size_t i = 0; i < b->n; i++)
            for (int c = 0; c < f; c++) final_values[i * f + c] = fin[i * 3 + c];
    return EFFSC_OK;
}

// Autotuner: time the batched protocol (one warm-up, then 3 replays each)
// over quadruples per thread {1, 2, 4, 8} x tail switch {off, 2^6, 2^8, 2^10,
// as large as shared memory allows}, keep the fastest, and append every
// measurement to cache_path (one JSON object per line) when it is given.
int effsc_batch_tune(effsc_batch* b, const effsc_transcript* const* transcripts, const char* cache_path,
                     int* quads_per_thread, uint64_t* tail_len) {
    if (!b || !transcripts) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    BCK(cudaSetDevice(b->device));
    const int qs[4] = {1, 2, 4, 8};
    const uint64_t tls[5] = {0, 1ULL << 6, 1ULL << 8, 1ULL << 10, ~0ULL};
    double best_ms = 1e30;
    int best_q = b->quads_per_thread;
    uint64_t best_t = b->tail_len;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    double times[5][4];
    for (int ti = 0; ti < 5; ti++)
        for (int k = 0; k < 4; k++) {
            b->quads_per_thread = qs[k];
            b->tail_len = tls[ti];
            int rc = plan(b);
            if (rc != EFFSC_OK) return rc;
            rc = effsc_batch_prove(b, transcripts, 1, nullptr, nullptr, nullptr);   // warm-up + capture
            if (rc != EFFSC_OK) return rc;
            float ms = 0;
            const int reps = 3;
            BCK(cudaEventRecord(e0, b->stream));
            for (int r = 0; r < reps; r++) {
                rc = effsc_batch_prove(b, transcripts, 1, nullptr, nullptr, nullptr);
                if (rc != EFFSC_OK) return rc;
            }
            BCK(cudaEventRecord(e1, b->stream));
            BCK(cudaEventSynchronize(e1));
            BCK(cudaEventElapsedTime(&ms, e0, e1));
            times[ti][k] = ms / reps;
            if (times[ti][k] < best_ms) { best_ms = times[ti][k]; best_q = qs[k]; best_t = tls[ti]; }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->quads_per_thread = best_q;
    b->tail_len = best_t;
    int rc = plan(b);
    if (rc != EFFSC_OK) return rc;
    if (quads_per_thread) *quads_per_thread = best_q;
    if (tail_len) *tail_len = best_t;
    if (cache_path && *cache_path) {
        FILE* fp = fopen(cache_path, "a");
        if (fp) {
            const int sms = max_grid() / 8;
            const u64 tmax = tail_max_len(b->pol, b->field == EFFSC_FP3 ? 3 : 1, TAIL_SMEM_CAP);
            fprintf(fp, "{\"kernel\": \"batch_round\", \"kind\": %d, \"field\": %d, \"instances\": %zu, "
                        "\"max_num_vars\": %u, \"sms\": %d, \"quads_per_thread\": %d, \"tail_len\": %llu, \"ms\": {",
                    b->kind, b->field, b->n, b->max_nv, sms, best_q,
                    (unsigned long long)std::min<uint64_t>(best_t, tmax));
            for (int ti = 0; ti < 5; ti++)
                for (int k = 0; k < 4; k++)
                    fprintf(fp, "%s\"q%d/tail%llu\": %.4f", (ti || k) ? ", " : "", qs[k],
                            (unsigned long long)std::min<uint64_t>(tls[ti], tmax), times[ti][k]);
            fprintf(fp, "}}\n");
            fclose(fp);
        }
    }
    return EFFSC_OK;
}

}  // extern "C"
