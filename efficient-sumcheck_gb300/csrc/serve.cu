// serve.cu -- a request loop that proves MSB InnerProduct / Multilinear
// sumchecks with continuous batching under an HBM budget.
//
// Requests queue on the host (FIFO).  Between steps the scheduler admits as
// many as the slot limit and the HBM budget allow: it reserves the request's
// device memory (tables, Fp3 work buffers, proof and transcript state) from
// the server's own stream-ordered pool, generates its tables or starts their
// upload on the lane's upload stream (a request with host tables joins the
// first step after they have arrived, so uploads overlap the steps) and
// writes its initial transcript state.  A step is ONE kernel launch in which
// every admitted request advances by one round -- whatever its kind, size or
// round -- or finalises; requests admitted while others are mid-proof join the
// next step.  A finished request's proof is copied to pinned host memory
// behind the step and its memory returned to the pool in stream order, so
// the next admission can reuse it at once.  Up to SERVE_INFLIGHT steps are
// queued ahead of the GPU; the host never waits on a step unless it must
// reuse that step's staging memory.
//
// Once a request's tables fit in one block's shared memory, its remaining
// rounds run in one tail launch (a block per request, on a second stream so
// they overlap the step) instead of one step each; its final fold joins the
// first step after the tail has finished.
//
// Each request's arithmetic, reductions and transcript are exactly those of
// the single-instance path (its own RoundArgs, grid-reduction counter and
// device transcript), so a proof does not depend on what else is in flight.
#include "effsc_gpu.h"
#include "kernels.h"
#include "keccak.cuh"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <deque>
#include <vector>

using namespace effsc;

void effsc_internal_tx_state(const effsc_transcript* t, void* out);
int effsc_internal_ctx_device(const effsc_ctx* c);
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c);
uint64_t effsc_internal_add_launches(uint64_t k);

#define SCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define TRYS(call)                           \
    do {                                     \
        const int rc_ = (call);              \
        if (rc_ != EFFSC_OK) return rc_;     \
    } while (0)

namespace {

constexpr int SERVE_INFLIGHT = 4;        // steps queued ahead of the GPU
constexpr u32 MAX_ROUNDS = 34;
constexpr size_t RES_WORDS = MAX_ROUNDS * 6 + MAX_ROUNDS * 3 + 3;   // wire | chal | final
constexpr size_t TX_WORDS = (sizeof(DevTranscript) + 7) / 8;

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    uint64_t id = 0;
    int kind = EFFSC_IP, field = EFFSC_FP3, ntab = 2;
    u32 n = 0;
    uint64_t seeds[2] = {0, 0};
    const uint64_t* htab[2] = {nullptr, nullptr};
    DevTranscript tx0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    size_t bytes = 0;
    // device
    u64* mem = nullptr;    // tables: per table 2^n input words then F3W * 2^(n-1) work words
    u64* res = nullptr;    // RES_WORDS proof words | transcript | counter
    u32 round = 0;         // next round (n: finalize)
    bool two_pass = false; // InnerProduct over Fp3, n >= 3: rounds 0-2 in two steps (ip01.cuh)
    bool in_tail = false;  // the remaining rounds are running in a tail launch
    cudaEvent_t tail_ev = nullptr;
    cudaEvent_t up_ev = nullptr;   // host tables: their upload on the lane's upload stream
    int slot = -1;         // pinned result slot
    cudaEvent_t ev = nullptr;
    u64* in(int t) const { return mem + (size_t)t * words_per_table(); }
    u64* work(int t) const { return in(t) + (1ULL << n); }
    size_t words_per_table() const { return (1ULL << n) + (size_t)(field == EFFSC_FP3 ? 3 : 1) * (1ULL << (n - 1)); }
    u64* wire() const { return res; }
    u64* chal() const { return res + MAX_ROUNDS * 6; }
    u64* fin() const { return res + MAX_ROUNDS * 9; }
    DevTranscript* tx() const { return (DevTranscript*)(res + RES_WORDS); }
    u32* counter() const { return (u32*)(res + RES_WORDS + TX_WORDS); }
};

struct Done {
    uint64_t id;
    int kind, field;
    u32 n;
    double t_submit, t_admit, t_done;
    std::vector<u64> out;   // RES_WORDS
};

size_t res_bytes() { return (RES_WORDS + TX_WORDS + 1) * sizeof(u64); }

}  // namespace

// Requests are split by size into two lanes, each with its own stream, FIFO
// queue, step staging and active set: a step of the small lane does not wait
// for the large requests' early rounds, and large requests do not block the
// admission of small ones.  Both lanes share the HBM budget, the slot limit,
// the memory pool and the result slots.
constexpr int SERVE_LANES = 2;
constexpr u32 SERVE_BIG_N = 22;   // requests of at least 2^22 entries per table: lane 1

struct Lane {
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaStream_t tail_stream = nullptr;
    cudaStream_t up_stream = nullptr;   // uploads of host tables, beside the steps
    std::deque<Req*> queue;
    std::vector<Req*> uploading;        // admitted, tables still crossing the host link
    std::vector<Req*> active;
    // step staging: pinned host + device copies of segments and args
    struct Stage {
        ServeSeg* h_segs = nullptr;
        RoundArgs* h_args = nullptr;
        DevTranscript* h_tx = nullptr;
        TailArgs* h_tail = nullptr;   // tail launches of the step (pinned)
        TailArgs* d_tail = nullptr;
        cudaEvent_t ev = nullptr;
        cudaEvent_t pre = nullptr;    // lane stream before the step's kernel
        cudaEvent_t tail_done = nullptr;
        bool busy = false, tail_busy = false;
    } stage[SERVE_INFLIGHT];
    int next_stage = 0;
    ServeSeg* d_segs = nullptr;
    RoundArgs* d_args = nullptr;
    u64* d_partials = nullptr;
};

struct effsc_server {
    effsc_ctx* ctx = nullptr;
    int device = 0;
    cudaMemPool_t pool = nullptr;
    uint64_t budget = 0, reserved = 0;
    u32 max_active = 0, n_active = 0;
    int quads_per_thread = 8;
    uint64_t next_id = 0;
    Lane lane[SERVE_LANES];
    std::deque<Req*> finishing;
    std::deque<Done> done;
    u32* h_status = nullptr;
    u32* d_status = nullptr;
    size_t partial_blocks = 0;
    // pinned result slots
    u64* h_results = nullptr;
    std::vector<int> free_slots;
    std::vector<cudaEvent_t> free_events;
    uint64_t steps = 0, kernels = 0;
};

namespace {

int deg_of_kind(int kind) { return kind == EFFSC_ML ? 1 : 2; }

size_t req_bytes(const Req& r) {
    return (size_t)r.ntab * r.words_per_table() * sizeof(u64) + res_bytes();
}

cudaEvent_t get_event(effsc_server* s) {
    if (!s->free_events.empty()) {
        cudaEvent_t e = s->free_events.back();
        s->free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

// Finished requests whose proof has reached host memory.
int retire(effsc_server* s, bool wait_one) {
    while (!s->finishing.empty()) {
        Req* r = s->finishing.front();
        cudaError_t q = wait_one ? cudaEventSynchronize(r->ev) : cudaEventQuery(r->ev);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "serving: %s", cudaGetErrorString(q));
        wait_one = false;
        if (*(volatile u32*)s->h_status) return effsc_set_error(EFFSC_TIMEOUT, "a serving step timed out");
        Done d;
        d.id = r->id;
        d.kind = r->kind;
        d.field = r->field;
        d.n = r->n;
        d.t_submit = r->t_submit;
        d.t_admit = r->t_admit;
        d.t_done = now_s();
        const u64* src = s->h_results + (size_t)r->slot * RES_WORDS;
        d.out.assign(src, src + RES_WORDS);
        s->done.push_back(std::move(d));
        s->free_slots.push_back(r->slot);
        s->free_events.push_back(r->ev);
        s->finishing.pop_front();
        delete r;
    }
    return EFFSC_OK;
}

// Admit the lane's queued requests (FIFO) while a slot and the HBM budget
// allow.  Initial transcript states go through the pinned staging of the
// lane's next step.
int activate(effsc_server* s, Lane& ln, Req* r, Lane::Stage& st, u32* ntx, std::vector<Req*>& fresh) {
    st.h_tx[*ntx] = r->tx0;
    (*ntx)++;
    fresh.push_back(r);
    r->round = 0;
    ln.active.push_back(r);
    return EFFSC_OK;
}

// Requests whose host tables have arrived join the next step.
int join_uploaded(effsc_server* s, Lane& ln, Lane::Stage& st, u32* ntx, std::vector<Req*>& fresh) {
    size_t keep = 0;
    for (size_t i = 0; i < ln.uploading.size(); i++) {
        Req* r = ln.uploading[i];
        const cudaError_t q = cudaEventQuery(r->up_ev);
        if (q == cudaErrorNotReady) { ln.uploading[keep++] = r; continue; }
        if (q != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "serving: %s", cudaGetErrorString(q));
        s->free_events.push_back(r->up_ev);
        r->up_ev = nullptr;
        TRYS(activate(s, ln, r, st, ntx, fresh));
    }
    ln.uploading.resize(keep);
    return EFFSC_OK;
}

int admit(effsc_server* s, Lane& ln, Lane::Stage& st, u32* ntx, std::vector<Req*>& fresh) {
    cudaStream_t cs = ln.stream;
    TRYS(join_uploaded(s, ln, st, ntx, fresh));
    while (!ln.queue.empty() && s->n_active < s->max_active) {
        Req* r = ln.queue.front();
        if (s->reserved + r->bytes > s->budget) break;
        void* mem = nullptr;
        void* res = nullptr;
        if (cudaMallocFromPoolAsync(&mem, (size_t)r->ntab * r->words_per_table() * sizeof(u64), s->pool, cs) != cudaSuccess ||
            cudaMallocFromPoolAsync(&res, res_bytes(), s->pool, cs) != cudaSuccess) {
            if (mem) cudaFreeAsync(mem, cs);
            cudaGetLastError();
            return effsc_set_error(EFFSC_OOM, "serving: device allocation of %zu bytes failed", r->bytes);
        }
        r->mem = (u64*)mem;
        r->res = (u64*)res;
        s->reserved += r->bytes;
        SCK(cudaMemsetAsync(r->counter(), 0, sizeof(u32), cs));
        r->t_admit = now_s();
        ln.queue.pop_front();
        s->n_active++;
        if (r->htab[0]) {
            // host tables cross the link on the upload stream (after the
            // allocation in the lane stream's order) while the steps run;
            // the request joins a step once they have arrived
            cudaEvent_t e = get_event(s);
            SCK(cudaEventRecord(e, cs));
            SCK(cudaStreamWaitEvent(ln.up_stream, e, 0));
            s->free_events.push_back(e);
            for (int t = 0; t < r->ntab; t++)
                SCK(cudaMemcpyAsync(r->in(t), r->htab[t], (1ULL << r->n) * sizeof(u64), cudaMemcpyHostToDevice,
                                    ln.up_stream));
            r->up_ev = get_event(s);
            SCK(cudaEventRecord(r->up_ev, ln.up_stream));
            ln.uploading.push_back(r);
            continue;
        }
        for (int t = 0; t < r->ntab; t++) launch_gen_uniform(r->seeds[t], 1ULL << r->n, r->in(t), cs);
        TRYS(activate(s, ln, r, st, ntx, fresh));
    }
    return EFFSC_OK;
}

// Current table length of a request about to run round `round`.
u64 req_len(const Req& r) { return r.round == 0 ? (1ULL << r.n) : (1ULL << (r.n - r.round + 1)); }

// The request's remaining rounds fit one tail launch: its tables fit in one
// block's shared memory (not in the middle of the two-pass start).
bool tail_eligible(const Req& r) {
    if (r.in_tail || r.round >= r.n) return false;
    if (r.two_pass && (r.round == 1 || r.round == 2)) return false;
    const int pol = r.kind == EFFSC_IP ? POL_IP : POL_ML, fw = r.field == EFFSC_FP3 ? 3 : 1;
    return req_len(r) <= tail_max_len(pol, fw, TAIL_SMEM_CAP);
}

void fill_tail(const Req& r, TailArgs& ta) {
    memset(&ta, 0, sizeof ta);
    const bool f3 = r.field == EFFSC_FP3;
    const int F3W = f3 ? 3 : 1;
    const u32 rd = r.round;
    const u64 half0 = 1ULL << (r.n - 1);
    ta.L = req_len(r);
    ta.nrounds = r.n - rd;
    ta.first_fold = rd ? 1 : 0;
    ta.chal_in = rd ? r.chal() + 3 * (rd - 1) : nullptr;
    ta.tx = r.tx();
    ta.proof_wire = r.wire() + (size_t)3 * deg_of_kind(r.kind) * rd;
    ta.proof_chal = r.chal() + 3 * rd;
    const u32 folds = ta.nrounds - (rd ? 0 : 1);
    for (int t = 0; t < r.ntab; t++) {
        if (rd <= 1) ta.in[t][0] = r.in(t);
        else {
            for (int c = 0; c < F3W; c++) ta.in[t][c] = r.work(t) + c * half0;
            if (f3) ta.in_ext |= 1u << t;
        }
        // the folded tables of length 2 go where the final fold reads them
        if (folds)
            for (int c = 0; c < F3W; c++) ta.out[t][c] = r.work(t) + c * half0;
    }
}

// One serving step of a lane: every active request runs its next round or
// finalises (or its remaining rounds start in a tail launch).
int step(effsc_server* s, Lane& ln) {
    cudaStream_t cs = ln.stream;
    Lane::Stage& st = ln.stage[ln.next_stage];
    if (st.busy) {
        SCK(cudaEventSynchronize(st.ev));
        st.busy = false;
    }
    if (st.tail_busy) {
        SCK(cudaEventSynchronize(st.tail_done));
        st.tail_busy = false;
    }
    u32 ntx = 0;
    std::vector<Req*> fresh;
    int rc = admit(s, ln, st, &ntx, fresh);
    if (rc != EFFSC_OK) return rc;
    // initial transcript states of the admitted requests: one H2D each from
    // the pinned stage (they are small and few)
    for (u32 k = 0; k < ntx; k++)
        SCK(cudaMemcpyAsync(fresh[k]->tx(), &st.h_tx[k], sizeof(DevTranscript), cudaMemcpyHostToDevice, cs));
    if (ln.active.empty()) return EFFSC_OK;
    const int maxb = max_grid();
    const u64 per_block = (u64)KERNEL_TPB * s->quads_per_thread;
    u32 first = 0, nseg = 0;
    std::vector<Req*> finals, tails;
    for (Req* r : ln.active) {
        if (r->in_tail) {
            const cudaError_t q = cudaEventQuery(r->tail_ev);
            if (q == cudaErrorNotReady) continue;   // still in its tail: nothing this step
            if (q != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "serving tail: %s", cudaGetErrorString(q));
            s->free_events.push_back(r->tail_ev);
            r->tail_ev = nullptr;
            r->in_tail = false;                      // round == n: the final fold below
        } else if (tail_eligible(*r)) {
            tails.push_back(r);
            continue;
        }
        const bool f3 = r->field == EFFSC_FP3;
        const int F3W = f3 ? 3 : 1;
        const int pol = r->kind == EFFSC_IP ? POL_IP : POL_ML;
        RoundArgs& a = st.h_args[nseg];
        memset(&a, 0, sizeof a);
        ServeSeg& sg = st.h_segs[nseg];
        sg.first_block = first;
        sg.reserved = 0;
        u32 code = (pol == POL_IP ? SERVE_IP : 0) | (f3 ? SERVE_FP3 : 0);
        const u64 half0 = 1ULL << (r->n - 1);
        const u32 rd = r->round;
        if (r->two_pass && rd < 3) {
            // rounds 0-1 from the base tables, then round 2 with the double fold
            const u64 L = 1ULL << r->n;
            code |= (rd == 0 ? SERVE_IP01 : SERVE_IP2X) << SERVE_PHASE_SHIFT;
            for (int t = 0; t < 2; t++) {
                a.t[t].in[0] = r->in(t);
                if (rd) for (int c = 0; c < 3; c++) a.t[t].out[c] = r->work(t) + c * half0;
            }
            a.L = L;
            a.chal_ptr = rd ? r->chal() : nullptr;
            a.chal2_ptr = rd ? r->chal() + 3 : nullptr;
            a.counter = r->counter();
            a.status = s->d_status;
            a.tx.tx = r->tx();
            a.tx.proof_wire = r->wire() + (size_t)6 * rd;
            a.tx.proof_chal = r->chal() + 3 * rd;
            const u64 work = rd == 0 ? L / 4 : L / 8;
            u64 nb = (work + per_block - 1) / per_block;
            nb = std::max<u64>(1, std::min<u64>(nb, (u64)maxb));
            sg.nblocks = (u32)nb;
        } else if (rd < r->n) {
            const u64 L = rd == 0 ? (1ULL << r->n) : (1ULL << (r->n - rd + 1));
            const u64 work = rd == 0 ? L / 2 : L / 4;
            const u32 phase = rd == 0 ? SERVE_EVAL : (rd == 1 || !f3) ? SERVE_FOLD_BASE : SERVE_FOLD_EXT;
            code |= phase << SERVE_PHASE_SHIFT;
            for (int t = 0; t < r->ntab; t++) {
                if (rd <= 1) a.t[t].in[0] = r->in(t);
                else for (int c = 0; c < F3W; c++) a.t[t].in[c] = r->work(t) + c * half0;
                if (rd >= 1)
                    for (int c = 0; c < F3W; c++) a.t[t].out[c] = r->work(t) + c * half0;
            }
            a.L = L;
            a.chal_ptr = rd ? r->chal() + 3 * (rd - 1) : nullptr;
            a.counter = r->counter();
            a.status = s->d_status;
            a.tx.tx = r->tx();
            a.tx.proof_wire = r->wire() + (size_t)3 * deg_of_kind(r->kind) * rd;
            a.tx.proof_chal = r->chal() + 3 * rd;
            u64 nb = (work + per_block - 1) / per_block;
            nb = std::max<u64>(1, std::min<u64>(nb, (u64)maxb));
            sg.nblocks = (u32)nb;
        } else {
            const bool ext = f3 && r->n >= 2;
            code |= (ext ? SERVE_FINAL_EXT : SERVE_FINAL_BASE) << SERVE_PHASE_SHIFT;
            for (int t = 0; t < r->ntab; t++) {
                if (r->n == 1) a.t[t].in[0] = r->in(t);
                else for (int c = 0; c < (ext ? 3 : 1); c++) a.t[t].in[c] = r->work(t) + c * half0;
            }
            a.chal_ptr = r->chal() + 3 * (r->n - 1);
            a.result = r->fin();
            sg.nblocks = 1;
            finals.push_back(r);
        }
        sg.code = code;
        first += sg.nblocks;
        nseg++;
    }
    if (first > s->partial_blocks) return effsc_set_error(EFFSC_INVALID_ARG, "serving step larger than planned");
    if (!tails.empty()) {
        // the tails depend on the requests' earlier rounds and admission
        // copies, all on the lane's stream before this point
        SCK(cudaEventRecord(st.pre, cs));
        SCK(cudaStreamWaitEvent(ln.tail_stream, st.pre, 0));
    }
    if (nseg) {
        for (u32 k = 0; k < nseg; k++) st.h_args[k].partials = ln.d_partials + (size_t)st.h_segs[k].first_block * 12;
        SCK(cudaMemcpyAsync(ln.d_segs, st.h_segs, nseg * sizeof(ServeSeg), cudaMemcpyHostToDevice, cs));
        SCK(cudaMemcpyAsync(ln.d_args, st.h_args, nseg * sizeof(RoundArgs), cudaMemcpyHostToDevice, cs));
        launch_serve_step(ln.d_segs, nseg, ln.d_args, first, cs);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "serving step launch: %s", cudaGetErrorString(e));
        s->kernels++;
        effsc_internal_add_launches(1);
    }
    s->steps++;
    if (!tails.empty()) {
        // one tail launch per (kind, field) group, a block per request
        cudaStream_t ts = ln.tail_stream;
        u32 nt = 0;
        for (int pol : {POL_IP, POL_ML})
            for (int fw : {1, 3}) {
                const u32 off = nt;
                u64 maxL = 0;
                for (Req* r : tails) {
                    if ((r->kind == EFFSC_IP ? POL_IP : POL_ML) != pol || (r->field == EFFSC_FP3 ? 3 : 1) != fw) continue;
                    fill_tail(*r, st.h_tail[nt]);
                    maxL = std::max<u64>(maxL, st.h_tail[nt].L);
                    nt++;
                }
                if (nt == off) continue;
                SCK(cudaMemcpyAsync(st.d_tail + off, st.h_tail + off, (nt - off) * sizeof(TailArgs), cudaMemcpyHostToDevice, ts));
                if (!launch_tail(pol, fw, st.d_tail + off, nullptr, nt - off, maxL, ts))
                    return effsc_set_error(EFFSC_CUDA_ERROR, "serving tail launch failed");
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "serving tail launch: %s", cudaGetErrorString(e));
                s->kernels++;
                effsc_internal_add_launches(1);
            }
        for (Req* r : tails) {
            r->tail_ev = get_event(s);
            SCK(cudaEventRecord(r->tail_ev, ts));
            r->in_tail = true;
            r->round = r->n;
        }
        SCK(cudaEventRecord(st.tail_done, ts));
        st.tail_busy = true;
    }
    // finished requests: proof to pinned memory, memory back to the pool
    for (Req* r : finals) {
        if (s->free_slots.empty()) {
            int rc2 = retire(s, true);
            if (rc2 != EFFSC_OK) return rc2;
            if (s->free_slots.empty()) return effsc_set_error(EFFSC_INVALID_ARG, "serving: no result slot");
        }
        r->slot = s->free_slots.back();
        s->free_slots.pop_back();
        SCK(cudaMemcpyAsync(s->h_results + (size_t)r->slot * RES_WORDS, r->res, RES_WORDS * sizeof(u64),
                            cudaMemcpyDeviceToHost, cs));
        r->ev = get_event(s);
        SCK(cudaEventRecord(r->ev, cs));
        SCK(cudaFreeAsync(r->mem, cs));
        SCK(cudaFreeAsync(r->res, cs));
        r->mem = nullptr;
        r->res = nullptr;
        s->reserved -= r->bytes;
        s->n_active--;
        s->finishing.push_back(r);
    }
    std::vector<Req*> still;
    still.reserve(ln.active.size());
    for (Req* r : ln.active) {
        if (r->in_tail) {
            still.push_back(r);            // its final fold comes after the tail
        } else if (r->round < r->n) {
            r->round += (r->two_pass && r->round == 0) ? 2 : 1;
            still.push_back(r);
        }
    }
    ln.active.swap(still);
    SCK(cudaEventRecord(st.ev, cs));
    st.busy = true;
    ln.next_stage = (ln.next_stage + 1) % SERVE_INFLIGHT;
    return EFFSC_OK;
}

size_t n_queued(const effsc_server* s) {
    size_t q = 0;
    for (const Lane& ln : s->lane) q += ln.queue.size();
    return q;
}

int submit_one(effsc_server* s, int kind, int field, uint32_t num_vars, const uint64_t* const* host_tables,
               const uint64_t* seeds, const effsc_transcript* t, double t_submit, uint64_t* id) {
    if (kind != EFFSC_IP && kind != EFFSC_ML) return effsc_set_error(EFFSC_UNSUPPORTED, "serving proves IP or ML requests");
    if (field != EFFSC_FP && field != EFFSC_FP3) return effsc_set_error(EFFSC_INVALID_ARG, "bad field");
    if (num_vars < 1 || num_vars > MAX_ROUNDS) return effsc_set_error(EFFSC_INVALID_ARG, "num_vars %u out of range 1..%u", num_vars, MAX_ROUNDS);
    if (!t || (!host_tables && !seeds)) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    Req* r = new Req();
    r->id = s->next_id++;
    r->kind = kind;
    r->field = field;
    r->ntab = kind == EFFSC_IP ? 2 : 1;
    r->n = num_vars;
    for (int k = 0; k < r->ntab; k++) {
        r->htab[k] = host_tables ? host_tables[k] : nullptr;
        r->seeds[k] = seeds ? seeds[k] : 0;
        if (host_tables && !host_tables[k]) { delete r; return effsc_set_error(EFFSC_INVALID_ARG, "table %d is NULL", k); }
    }
    effsc_internal_tx_state(t, &r->tx0);
    if ((int)r->tx0.deg != field) { delete r; return effsc_set_error(EFFSC_INVALID_ARG, "transcript: wrong field or kind"); }
    r->two_pass = kind == EFFSC_IP && field == EFFSC_FP3 && num_vars >= 3;
    r->bytes = req_bytes(*r);
    if (r->bytes > s->budget) {
        size_t b = r->bytes;
        delete r;
        return effsc_set_error(EFFSC_INVALID_ARG, "request needs %zu bytes, more than the HBM budget", b);
    }
    r->t_submit = t_submit;
    s->lane[num_vars >= SERVE_BIG_N ? 1 : 0].queue.push_back(r);
    if (id) *id = r->id;
    return EFFSC_OK;
}

// Proof rows out: `out_deg` elements per row of round_polys (the request's
// degree, or 2 for the trace layout, padded with zeros).
void copy_out(const Done& d, int out_deg, uint64_t* round_polys, uint64_t* challenges, uint64_t* final_value) {
    const int dg = deg_of_kind(d.kind), f = d.field;
    for (u32 row = 0; row < d.n; row++) {
        if (round_polys)
            for (int k = 0; k < out_deg; k++)
                for (int c = 0; c < f; c++)
                    round_polys[((size_t)row * out_deg + k) * f + c] = k < dg ? d.out[((size_t)row * dg + k) * 3 + c] : 0;
        if (challenges)
            for (int c = 0; c < f; c++) challenges[(size_t)row * f + c] = d.out[MAX_ROUNDS * 6 + row * 3 + c];
    }
    if (final_value)
        for (int c = 0; c < f; c++) final_value[c] = d.out[MAX_ROUNDS * 9 + c];
}

}  // namespace

extern "C" {

int effsc_server_create(effsc_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t max_active, effsc_server** out) {
    if (!ctx || !out || !hbm_budget_bytes || !max_active || max_active > 4096)
        return effsc_set_error(EFFSC_INVALID_ARG, "bad server arguments");
    SCK(cudaSetDevice(effsc_internal_ctx_device(ctx)));
    effsc_server* s = new effsc_server();
    s->ctx = ctx;
    s->device = effsc_internal_ctx_device(ctx);
    s->budget = hbm_budget_bytes;
    s->max_active = max_active;
    auto bail = [&](int rc) { effsc_server_destroy(s); return rc; };
    cudaMemPoolProps props;
    memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess)
        return bail(effsc_set_error(EFFSC_CUDA_ERROR, "serving: memory pool creation failed"));
    uint64_t keep = ~0ULL;   // keep freed memory in the pool for the next admissions
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    s->partial_blocks = (size_t)max_active * max_grid();
    for (int l = 0; l < SERVE_LANES; l++) {
        Lane& ln = s->lane[l];
        if (l == 0) ln.stream = effsc_internal_ctx_stream(ctx);
        else if (cudaStreamCreateWithFlags(&ln.stream, cudaStreamNonBlocking) != cudaSuccess)
            return bail(effsc_set_error(EFFSC_CUDA_ERROR, "serving: stream creation failed"));
        else ln.own_stream = true;
        if (cudaStreamCreateWithFlags(&ln.tail_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&ln.up_stream, cudaStreamNonBlocking) != cudaSuccess)
            return bail(effsc_set_error(EFFSC_CUDA_ERROR, "serving: stream creation failed"));
        for (int k = 0; k < SERVE_INFLIGHT; k++) {
            Lane::Stage& st = ln.stage[k];
            if (cudaHostAlloc((void**)&st.h_segs, max_active * sizeof(ServeSeg), cudaHostAllocDefault) != cudaSuccess ||
                cudaHostAlloc((void**)&st.h_args, max_active * sizeof(RoundArgs), cudaHostAllocDefault) != cudaSuccess ||
                cudaHostAlloc((void**)&st.h_tx, max_active * sizeof(DevTranscript), cudaHostAllocDefault) != cudaSuccess ||
                cudaHostAlloc((void**)&st.h_tail, max_active * sizeof(TailArgs), cudaHostAllocDefault) != cudaSuccess ||
                cudaMalloc((void**)&st.d_tail, max_active * sizeof(TailArgs)) != cudaSuccess ||
                cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&st.pre, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&st.tail_done, cudaEventDisableTiming) != cudaSuccess)
                return bail(effsc_set_error(EFFSC_OOM, "serving: pinned staging allocation failed"));
        }
        if (cudaMalloc((void**)&ln.d_segs, max_active * sizeof(ServeSeg)) != cudaSuccess ||
            cudaMalloc((void**)&ln.d_args, max_active * sizeof(RoundArgs)) != cudaSuccess ||
            cudaMalloc((void**)&ln.d_partials, s->partial_blocks * 12 * sizeof(u64)) != cudaSuccess)
            return bail(effsc_set_error(EFFSC_OOM, "serving: allocation failed"));
    }
    const size_t nslots = (size_t)2 * max_active * SERVE_INFLIGHT;
    if (cudaHostAlloc((void**)&s->h_results, nslots * RES_WORDS * sizeof(u64), cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&s->h_status, sizeof(u32), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->d_status, s->h_status, 0) != cudaSuccess)
        return bail(effsc_set_error(EFFSC_OOM, "serving: allocation failed"));
    *s->h_status = 0;
    for (size_t k = 0; k < nslots; k++) s->free_slots.push_back((int)(nslots - 1 - k));
    *out = s;
    return EFFSC_OK;
}

int effsc_server_destroy(effsc_server* s) {
    if (!s) return EFFSC_OK;
    cudaSetDevice(s->device);
    for (Lane& ln : s->lane) {
        if (ln.up_stream) cudaStreamSynchronize(ln.up_stream);
        if (ln.tail_stream) cudaStreamSynchronize(ln.tail_stream);
        if (ln.stream) cudaStreamSynchronize(ln.stream);
    }
    for (Lane& ln : s->lane) {
        for (Req* r : ln.uploading) ln.active.push_back(r);
        ln.uploading.clear();
        for (Req* r : ln.active) {
            if (r->up_ev) cudaEventDestroy(r->up_ev);
            if (r->mem) cudaFreeAsync(r->mem, ln.stream);
            if (r->res) cudaFreeAsync(r->res, ln.stream);
            if (r->tail_ev) cudaEventDestroy(r->tail_ev);
            delete r;
        }
        for (Req* r : ln.queue) delete r;
        if (ln.stream) cudaStreamSynchronize(ln.stream);
    }
    for (Req* r : s->finishing) { if (r->ev) cudaEventDestroy(r->ev); delete r; }
    for (cudaEvent_t e : s->free_events) cudaEventDestroy(e);
    for (Lane& ln : s->lane) {
        for (int k = 0; k < SERVE_INFLIGHT; k++) {
            Lane::Stage& st = ln.stage[k];
            if (st.h_segs) cudaFreeHost(st.h_segs);
            if (st.h_args) cudaFreeHost(st.h_args);
            if (st.h_tx) cudaFreeHost(st.h_tx);
            if (st.h_tail) cudaFreeHost(st.h_tail);
            if (st.d_tail) cudaFree(st.d_tail);
            if (st.ev) cudaEventDestroy(st.ev);
            if (st.pre) cudaEventDestroy(st.pre);
            if (st.tail_done) cudaEventDestroy(st.tail_done);
        }
        if (ln.d_segs) cudaFree(ln.d_segs);
        if (ln.d_args) cudaFree(ln.d_args);
        if (ln.d_partials) cudaFree(ln.d_partials);
        if (ln.tail_stream) cudaStreamDestroy(ln.tail_stream);
        if (ln.up_stream) cudaStreamDestroy(ln.up_stream);
        if (ln.own_stream) cudaStreamDestroy(ln.stream);
    }
    if (s->h_results) cudaFreeHost(s->h_results);
    if (s->h_status) cudaFreeHost(s->h_status);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return EFFSC_OK;
}

int effsc_server_submit(effsc_server* s, int kind, int field, uint32_t num_vars, const uint64_t* const* host_tables,
                        const uint64_t* seeds, const effsc_transcript* t, uint64_t* id) {
    if (!s) return effsc_set_error(EFFSC_INVALID_ARG, "NULL server");
    return submit_one(s, kind, field, num_vars, host_tables, seeds, t, now_s(), id);
}

int effsc_server_progress(effsc_server* s, int wait, uint32_t* pending) {
    if (!s) return effsc_set_error(EFFSC_INVALID_ARG, "NULL server");
    SCK(cudaSetDevice(s->device));
    int rc = retire(s, false);
    if (rc != EFFSC_OK) return rc;
    for (Lane& ln : s->lane)
        if (!ln.active.empty() || !ln.queue.empty() || !ln.uploading.empty()) {
            rc = step(s, ln);
            if (rc != EFFSC_OK) return rc;
        }
    if (wait && s->done.empty() && !s->finishing.empty()) {
        rc = retire(s, true);
        if (rc != EFFSC_OK) return rc;
    }
    if (pending) *pending = (uint32_t)(n_queued(s) + s->n_active + s->finishing.size());
    return EFFSC_OK;
}

int effsc_server_take(effsc_server* s, uint64_t* id, uint32_t* num_vars, uint64_t* round_polys, uint64_t* challenges,
                      uint64_t* final_value, double* queue_s, double* latency_s) {
    if (!s || !id) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    if (s->done.empty()) { *id = ~0ULL; return EFFSC_OK; }
    const Done& d = s->done.front();
    *id = d.id;
    if (num_vars) *num_vars = d.n;
    copy_out(d, deg_of_kind(d.kind), round_polys, challenges, final_value);
    if (queue_s) *queue_s = d.t_admit - d.t_submit;
    if (latency_s) *latency_s = d.t_done - d.t_submit;
    s->done.pop_front();
    return EFFSC_OK;
}

}  // extern "C"

// The open-loop driver behind both trace entry points: request i's tables
// come from seeds[2i..2i+1] or, with seeds NULL, from host_tables[2i..2i+1].
static int run_trace_impl(effsc_server* s, size_t n, const int* kinds, int field, const uint32_t* num_vars,
                          const uint64_t* seeds, const uint64_t* const* host_tables,
                          const effsc_transcript* const* transcripts, const double* arrival_s, double* latency_s,
                          double* makespan_s, uint64_t* round_polys, uint64_t* challenges, uint64_t* final_values) {
    if (!s || !kinds || !num_vars || (!seeds && !host_tables) || !transcripts || !arrival_s || !latency_s)
        return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    if (n_queued(s) || s->n_active || !s->finishing.empty() || !s->done.empty())
        return effsc_set_error(EFFSC_INVALID_ARG, "run_trace needs an idle server");
    SCK(cudaSetDevice(s->device));
    std::vector<size_t> row(n + 1, 0), order(n);
    for (size_t i = 0; i < n; i++) {
        row[i + 1] = row[i] + num_vars[i];
        order[i] = i;
    }
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return arrival_s[x] < arrival_s[y]; });
    std::vector<size_t> of_id;   // request id -> trace index
    const uint64_t id0 = s->next_id;
    const double t0 = now_s();
    size_t next = 0, finished = 0;
    while (finished < n) {
        const double t = now_s() - t0;
        while (next < n && arrival_s[order[next]] <= t) {
            const size_t i = order[next];
            uint64_t id;
            int rc = submit_one(s, kinds[i], field, num_vars[i], seeds ? nullptr : host_tables + 2 * i,
                                seeds ? seeds + 2 * i : nullptr, transcripts[i], t0 + arrival_s[i], &id);
            if (rc != EFFSC_OK) return rc;
            if (of_id.size() <= id - id0) of_id.resize(id - id0 + 1);
            of_id[id - id0] = i;
            next++;
        }
        const bool idle = !n_queued(s) && !s->n_active;
        if (!idle) {
            int rc = effsc_server_progress(s, 0, nullptr);
            if (rc != EFFSC_OK) return rc;
        } else {
            int rc = retire(s, false);
            if (rc != EFFSC_OK) return rc;
        }
        while (!s->done.empty()) {
            const Done& d = s->done.front();
            const size_t i = of_id[d.id - id0];
            copy_out(d, 2, round_polys ? round_polys + row[i] * 2 * field : nullptr,
                     challenges ? challenges + row[i] * field : nullptr,
                     final_values ? final_values + i * field : nullptr);
            latency_s[i] = d.t_done - d.t_submit;
            s->done.pop_front();
            finished++;
        }
        if (idle && s->finishing.empty() && next < n) {
            // nothing on the GPU: wait for the next arrival
            while (now_s() - t0 < arrival_s[order[next]]) {}
        }
    }
    if (makespan_s) *makespan_s = now_s() - t0;
    return EFFSC_OK;
}

extern "C" {

int effsc_server_run_trace(effsc_server* s, size_t n, const int* kinds, int field, const uint32_t* num_vars,
                           const uint64_t* seeds, const effsc_transcript* const* transcripts, const double* arrival_s,
                           double* latency_s, double* makespan_s, uint64_t* round_polys, uint64_t* challenges,
                           uint64_t* final_values) {
    if (!seeds) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    return run_trace_impl(s, n, kinds, field, num_vars, seeds, nullptr, transcripts, arrival_s, latency_s,
                          makespan_s, round_polys, challenges, final_values);
}

int effsc_server_run_trace_host(effsc_server* s, size_t n, const int* kinds, int field, const uint32_t* num_vars,
                                const uint64_t* const* host_tables, const effsc_transcript* const* transcripts,
                                const double* arrival_s, double* latency_s, double* makespan_s, uint64_t* round_polys,
                                uint64_t* challenges, uint64_t* final_values) {
    if (!host_tables) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    return run_trace_impl(s, n, kinds, field, num_vars, nullptr, host_tables, transcripts, arrival_s, latency_s,
                          makespan_s, round_polys, challenges, final_values);
}

}  // extern "C"
