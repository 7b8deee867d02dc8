// k_tail.cu -- the tail rounds of an MSB Multilinear / InnerProduct proof in
// one thread block.
//
// Once a prover's tables are small, a round costs far more in kernel
// boundaries (launch, grid-wide ticket, a lone last block running the
// transcript) than in arithmetic.  The tail kernel loads the tables into
// shared memory once (base tables embedded when the field is Fp3), then per
// round: folds in place with the previous challenge (new = lo + (hi - lo) r,
// reference src/inner_product_sumcheck.rs:143-176 and
// src/multilinear_sumcheck.rs:132-178), accumulates the round polynomial of
// the folded tables on the fly (the same quadruple scheme as the fused
// kernels), reduces across the block, and runs the transcript step (wire
// values, hook bytes, challenge squeeze) in warp 0.  After the
// last round the folded tables go back to global memory so that finalize /
// final_value and the post-state accessors see exactly what the per-round
// path would leave.  A batch launches one block per instance.
#include "round_common.cuh"

#include <atomic>
#include <cstring>

namespace effsc {

template <int FW>
__device__ __forceinline__ F3 sm_ld(const u64* sm, u64 L, int t, u64 i) {
    F3 r;
    r.c0 = sm[(u64)(t * FW) * L + i];
    if (FW == 3) { r.c1 = sm[(u64)(t * 3 + 1) * L + i]; r.c2 = sm[(u64)(t * 3 + 2) * L + i]; }
    else { r.c1 = r.c2 = 0; }
    return r;
}
template <int FW>
__device__ __forceinline__ void sm_st(u64* sm, u64 L, int t, u64 i, const F3& v) {
    sm[(u64)(t * FW) * L + i] = v.c0;
    if (FW == 3) { sm[(u64)(t * 3 + 1) * L + i] = v.c1; sm[(u64)(t * 3 + 2) * L + i] = v.c2; }
}

constexpr int TAIL_TPB = 512;
constexpr int TAIL_NW = TAIL_TPB / 32;

// Index i of a table of 2^lg entries with its lg bits reversed.  An LSB
// prover's table held in this order makes its folds (2j, 2j+1) -> j MSB
// folds (p, p + L/2) -> p, in place, with entry j of every later length at
// the reversed position again; so the LSB tail is the MSB tail on a
// bit-reversed layout, reversed back when the tables are written out.
__device__ __forceinline__ u64 tail_rev(u64 i, u32 lg) { return lg ? (u64)(__brev((u32)i) >> (32 - lg)) : 0; }
__device__ __forceinline__ u32 tail_lg(u64 n) { return n > 1 ? 63 - __clzll(n) : 0; }

// Shared state of a tail block: block partials, round totals, challenge,
// squeeze scratch, and (cluster kernel, CTA 0) the partials of every CTA.
constexpr int TAIL_NW3 = 12;
constexpr int TAIL_MAX_CS = 16;
struct TailShared {
    u64 red[TAIL_NW][TAIL_NW3];
    u64 tot[TAIL_NW3];
    u64 chal[3];
    __align__(8) uint8_t scr[64];
    u64 cred[TAIL_MAX_CS][TAIL_NW3];
};

// Fold (pairs q, q+2Q and q+Q, q+3Q of the quarter length Q) and accumulate
// the round polynomial of the folded tables; `put` stores the folded pair.
template <int POL, int FW, class Put>
__device__ __forceinline__ void tail_fold_eval(const u64* smb, u64 stride, u64 len, const u64* chal,
                                               Policy<POL, FW == 3 ? (1u << Policy<POL, 0>::NT) - 1 : 0>& acc, Put put) {
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr bool E = FW == 3;
    const Mul3 m = mul3_prepare<E>(f3_make(chal[0], chal[1], chal[2]));
    const u64 Q = len >> 2;
    F3 lo[NT], hi[NT];
    for (u64 q = threadIdx.x; q < Q; q += TAIL_TPB) {
#pragma unroll
        for (int t = 0; t < NT; t++) {
            F3 x0 = sm_ld<FW>(smb, stride, t, q), x1 = sm_ld<FW>(smb, stride, t, q + Q);
            F3 x2 = sm_ld<FW>(smb, stride, t, q + 2 * Q), x3 = sm_ld<FW>(smb, stride, t, q + 3 * Q);
            lo[t] = f3_fold<E, E>(x0, x2, m);
            hi[t] = f3_fold<E, E>(x1, x3, m);
            put(t, q, Q, lo[t], hi[t]);
        }
        acc.pair(lo, hi);
    }
}

// Block reduction of the round polynomial into sh.tot (lanes < NW3 of warp 0).
template <int NRAW>
__device__ __forceinline__ void tail_block_reduce(F3* raw, bool active, TailShared& sh) {
    constexpr int NW3 = 3 * NRAW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (active) {
#pragma unroll
        for (int off = 16; off; off >>= 1) {
#pragma unroll
            for (int i = 0; i < NRAW; i++) {
                raw[i].c0 = gl_add(raw[i].c0, __shfl_down_sync(0xffffffffu, raw[i].c0, off));
                raw[i].c1 = gl_add(raw[i].c1, __shfl_down_sync(0xffffffffu, raw[i].c1, off));
                raw[i].c2 = gl_add(raw[i].c2, __shfl_down_sync(0xffffffffu, raw[i].c2, off));
            }
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NRAW; i++) { sh.red[warp][3 * i] = raw[i].c0; sh.red[warp][3 * i + 1] = raw[i].c1; sh.red[warp][3 * i + 2] = raw[i].c2; }
    }
    __syncthreads();
    if (warp == 0 && lane < NW3) {
        u64 v = 0;
#pragma unroll
        for (int q = 0; q < TAIL_NW; q++) v = gl_add(v, sh.red[q][lane]);
        sh.tot[lane] = v;
    }
}

// Transcript step of round k in warp 0 (src/runner.rs:39-55): send the wire
// values in sh.tot, absorb the hook, squeeze the challenge into sh.chal and
// record both in the proof.
template <int POL>
__device__ __forceinline__ void tail_transcript(WarpTx& w, const TailArgs& a, u32 k, TailShared& sh) {
    constexpr int NWIRE = POL == POL_ML ? 1 : 2;
    const int lane = threadIdx.x & 31;
    tx_send_elems(w, lane, sh.tot, NWIRE);
    if (a.hook_len) {
        const uint8_t* hk = a.hook;
        if (((w.pos & 7) == 0 || w.squeezing) && (a.hook_len & 7) == 0 && ((uintptr_t)hk & 7) == 0) {
            const u64* hw = (const u64*)hk;
            tx_absorb_words(w, lane, a.hook_len >> 3, [&](u32 i) -> u64 { return hw[i]; });
        } else {
            tx_absorb(w, lane, a.hook_len, [&](u32 i) -> uint8_t { return hk[i]; });
        }
    }
    tx_challenge(w, lane, sh.chal, sh.scr);
    if (lane < 3 * NWIRE) a.proof_wire[(u64)k * 3 * NWIRE + lane] = sh.tot[lane];
    if (lane < 3) a.proof_chal[(u64)k * 3 + lane] = sh.chal[lane];
}

// After the last round: store the transcript state, apply the runner's
// finalize fold, write the read-back entries and the folded tables.
template <int POL, int FW>
__device__ __forceinline__ void tail_finish(u64* smb, u64 stride, u64 len, const TailArgs& a, WarpTx& w, TailShared& sh) {
    constexpr int NT = Policy<POL, 0>::NT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) tx_store((DevTranscript*)a.tx, w, lane);
    if (a.final_fold && len >= 2) {
        // SumcheckProver::finalize with the last challenge: one MSB fold
        // (src/inner_product_sumcheck.rs:143-176, src/multilinear_sumcheck.rs:132-178)
        constexpr bool E = FW == 3;
        const Mul3 m = mul3_prepare<E>(f3_make(sh.chal[0], sh.chal[1], sh.chal[2]));
        const u64 half = len >> 1;
        for (u64 j = threadIdx.x; j < half; j += TAIL_TPB)
#pragma unroll
            for (int t = 0; t < NT; t++)
                sm_st<FW>(smb, stride, t, j, f3_fold<E, E>(sm_ld<FW>(smb, stride, t, j), sm_ld<FW>(smb, stride, t, j + half), m));
        __syncthreads();
        len = half;
    }
    if (a.first_out && threadIdx.x < 12) {
        const int t = threadIdx.x / 3, c = threadIdx.x % 3;
        a.first_out[threadIdx.x] = (t < NT && c < FW) ? smb[(u64)(t * FW + c) * stride] : 0;
    }
    // write back the tables after the last fold (LSB: from the reversed layout)
    if (a.out[0][0]) {
        const u32 lg = tail_lg(len);
        for (int t = 0; t < NT; t++)
            for (int c = 0; c < FW; c++) {
                const u64* src = smb + (u64)(t * FW + c) * stride;
                u64* dst = a.out[t][c];
                for (u64 i = threadIdx.x; i < len; i += TAIL_TPB) dst[i] = src[a.lsb ? tail_rev(i, lg) : i];
            }
    }
}

// Rounds k0 .. a.nrounds-1 in one block on tables of length `len` at smb
// (table t, component c, element i at smb[(t*FW + c)*stride + i]); then the
// folded tables go back to global memory and the transcript state is stored.
template <int POL, int FW>
__device__ void tail_loop(u64* smb, u64 stride, u64 len, u32 k0, bool fold, const TailArgs& a, WarpTx& w,
                          TailShared& sh) {
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 MF = FW == 3 ? (1u << NT) - 1 : 0;
    using P = Policy<POL, MF>;
    const int warp = threadIdx.x >> 5;
    for (u32 k = k0; k < a.nrounds; k++) {
        // warps without entries this round skip the arithmetic and the
        // reduction of their (zero) sums; every warp reaches both barriers
        const u64 nwork = fold ? (len >> 2) : len == 1 ? 1 : (len >> 1);
        const bool active = (u64)warp * 32 < nwork;
        P acc;
        F3 raw[P::NRAW];
#pragma unroll
        for (int i = 0; i < P::NRAW; i++) raw[i] = f3_zero();
        if (active) {
            acc.init();
            F3 lo[NT], hi[NT];
            if (fold) {
                tail_fold_eval<POL, FW>(smb, stride, len, sh.chal, acc, [&](int t, u64 q, u64 Q, const F3& l, const F3& h) {
                    sm_st<FW>(smb, stride, t, q, l);
                    sm_st<FW>(smb, stride, t, q + Q, h);
                });
            } else if (len == 1) {
                if (threadIdx.x == 0) {
#pragma unroll
                    for (int t = 0; t < NT; t++) lo[t] = sm_ld<FW>(smb, stride, t, 0);
                    acc.single(lo);
                }
            } else {
                const u64 half = len >> 1;
                for (u64 j = threadIdx.x; j < half; j += TAIL_TPB) {
#pragma unroll
                    for (int t = 0; t < NT; t++) { lo[t] = sm_ld<FW>(smb, stride, t, j); hi[t] = sm_ld<FW>(smb, stride, t, j + half); }
                    acc.pair(lo, hi);
                }
            }
            acc.result(raw);
        }
        if (fold) len >>= 1;
        tail_block_reduce<P::NRAW>(raw, active, sh);
        if (warp == 0) {
            __syncwarp();
            tail_transcript<POL>(w, a, k, sh);
        }
        __syncthreads();
        fold = true;
    }
    tail_finish<POL, FW>(smb, stride, len, a, w, sh);
}

// Shared-memory layout: table t, component c, element i at sm[(t*FW + c)*L0 + i]
// with L0 the starting length (rows keep their stride as the tables shrink).
// Warp 0 keeps the transcript state in registers for the whole tail and the
// challenge stays in shared memory, so a round costs one block reduction and
// one transcript step.
template <int POL, int FW>
__device__ void tail_body(const TailArgs& a) {
    extern __shared__ __align__(16) u64 sm[];
    constexpr int NT = Policy<POL, 0>::NT;
    __shared__ TailShared sh;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 L0 = a.L;
    const u32 lg0 = tail_lg(L0);
    for (int t = 0; t < NT; t++)
        for (int c = 0; c < FW; c++) {
            const u64* src = (c == 0 || ((a.in_ext >> t) & 1u)) ? a.in[t][c] : nullptr;
            u64* dst = sm + (u64)(t * FW + c) * L0;
            for (u64 i = threadIdx.x; i < L0; i += TAIL_TPB) dst[a.lsb ? tail_rev(i, lg0) : i] = src ? src[i] : 0;
        }
    if (threadIdx.x < 3) sh.chal[threadIdx.x] = a.first_fold ? a.chal_in[threadIdx.x] : 0;
    WarpTx w;
    if (warp == 0) w = tx_load((const DevTranscript*)a.tx, lane);
    __syncthreads();
    tail_loop<POL, FW>(sm, L0, L0, 0, a.first_fold != 0, a, w, sh);
}

// ---- cluster tail ---------------------------------------------------------
// Tables up to CS times one block's capacity: a thread-block cluster of CS
// CTAs holds them in distributed shared memory, CTA c the groups of G = 16
// consecutive entries whose group index is c mod CS: entry k with
// (k / G) mod CS = c at local index (k / (G CS)) G + k mod G.  The slices
// load as whole 128-byte lines, and MSB pairs (k, k + L/2) are local pairs
// (j, j + L/(2 CS)) while L/2 is a multiple of G CS, so each CTA folds and
// evaluates its slice exactly as the one-block tail does; the CTAs' sums meet in CTA 0 (distributed
// shared memory stores), which runs the transcript step and writes the
// challenge back into every CTA.  After log2(CS) + 1 rounds the last fold
// writes the table (now half a slice long) straight into CTA 0, which
// finishes the proof alone.  Every CTA passes the same 1 + 2 (log2(CS) + 1)
// cluster barriers.
constexpr u64 CL_G = 16;
// Global index of local entry j of CTA c.
__device__ __forceinline__ u64 cl_global(u64 j, u32 c, u32 cs_log) {
    return (((j / CL_G) << cs_log) + c) * CL_G + (j % CL_G);
}
__device__ __forceinline__ u32 cluster_rank() {
    u32 r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Store v at the shared-memory location p of CTA `rank` in the cluster.
__device__ __forceinline__ void dsmem_st(const void* p, u32 rank, u64 v) {
    u32 remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(smem_u32(p)), "r"(rank));
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(remote), "l"(v) : "memory");
}

// The H = log2(CS) + 1 cluster rounds of k_tail_cluster as separate loops
// (Multilinear: its cheap rounds measured faster this way, with CTA 0 going
// on in tail_loop, than in the one loop InnerProduct uses: n = 20, 168
// against 178 us per proof); the last fold hands the table to CTA 0.
template <int POL, int FW>
__device__ __forceinline__ void tail_cluster_rounds(u64* sm, u64 Ll, u64& len, u32 cs_log, u32 rank, const TailArgs& a,
                                                    WarpTx& w, TailShared& sh) {
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 MF = FW == 3 ? (1u << NT) - 1 : 0;
    using P = Policy<POL, MF>;
    constexpr int NW3 = 3 * P::NRAW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u32 CS = 1u << cs_log, H = cs_log + 1;
    for (u32 k = 0; k < H; k++) {
        const u64 ll = len >> cs_log;      // slice length this round (>= 4)
        const bool last = k + 1 == H;
        P acc;
        acc.init();
        F3 raw[P::NRAW];
        if (!last) {
            tail_fold_eval<POL, FW>(sm, Ll, ll, sh.chal, acc, [&](int t, u64 q, u64 Q, const F3& l, const F3& h) {
                sm_st<FW>(sm, Ll, t, q, l);
                sm_st<FW>(sm, Ll, t, q + Q, h);
            });
        } else {
            // the folded table (L0 / 2^H = Ll / 2 entries) goes to CTA 0's
            // rows from offset Ll / 2 on, at its global index
            tail_fold_eval<POL, FW>(sm, Ll, ll, sh.chal, acc, [&](int t, u64 q, u64 Q, const F3& l, const F3& h) {
                const u64 g_lo = cl_global(q, rank, cs_log), g_hi = cl_global(q + Q, rank, cs_log);
                u64* row = sm + (u64)(t * FW) * Ll + Ll / 2;
                dsmem_st(row + g_lo, 0, l.c0);
                dsmem_st(row + g_hi, 0, h.c0);
                if (FW == 3) {
                    dsmem_st(row + Ll + g_lo, 0, l.c1);
                    dsmem_st(row + Ll + g_hi, 0, h.c1);
                    dsmem_st(row + 2 * Ll + g_lo, 0, l.c2);
                    dsmem_st(row + 2 * Ll + g_hi, 0, h.c2);
                }
            });
        }
        acc.result(raw);
        len >>= 1;
        tail_block_reduce<P::NRAW>(raw, true, sh);
        if (warp == 0 && lane < NW3) dsmem_st(&sh.cred[rank][lane], 0, sh.tot[lane]);
        cluster_sync_all();   // all CTAs' sums (and in the last round the table) are in CTA 0
        if (rank == 0 && warp == 0) {
            if (lane < NW3) {
                u64 v = 0;
                for (u32 c = 0; c < CS; c++) v = gl_add(v, sh.cred[c][lane]);
                sh.tot[lane] = v;
            }
            __syncwarp();
            tail_transcript<POL>(w, a, k, sh);
            __syncwarp();
            if (lane >= 1 && (u32)lane < CS)
                for (int c = 0; c < 3; c++) dsmem_st(&sh.chal[c], (u32)lane, sh.chal[c]);
        }
        cluster_sync_all();   // the challenge is in every CTA
    }
}

template <int POL, int FW>
__global__ void __launch_bounds__(TAIL_TPB, 1) k_tail_cluster(TailArgs a, u32 cs_log) {
    extern __shared__ __align__(16) u64 sm[];
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 MF = FW == 3 ? (1u << NT) - 1 : 0;
    using P = Policy<POL, MF>;
    constexpr int NW3 = 3 * P::NRAW;
    __shared__ TailShared sh;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u32 CS = 1u << cs_log, rank = cluster_rank();
    const u64 L0 = a.L, Ll = L0 >> cs_log;   // slice length (row stride)
    // this CTA's slice; base tables are embedded when the field is Fp3
    for (int t = 0; t < NT; t++)
        for (int c = 0; c < FW; c++) {
            const u64* src = (c == 0 || ((a.in_ext >> t) & 1u)) ? a.in[t][c] : nullptr;
            u64* dst = sm + (u64)(t * FW + c) * Ll;
            for (u64 j = threadIdx.x; j < Ll; j += TAIL_TPB) dst[j] = src ? src[cl_global(j, rank, cs_log)] : 0;
        }
    if (threadIdx.x < 3) sh.chal[threadIdx.x] = a.chal_in[threadIdx.x];
    WarpTx w;
    if (rank == 0 && warp == 0) w = tx_load((const DevTranscript*)a.tx, lane);
    cluster_sync_all();   // every CTA is running before any remote store
    // InnerProduct: every round runs the same loop body, the cluster rounds
    // (k < H) and CTA 0's rounds after them -- one copy of the fold,
    // reduction and transcript code, already in the SM's instruction cache
    // when CTA 0 goes on alone (a separate copy measured ~15 us for CTA 0's
    // first round against ~3 us for the next ones; n = 26: 0.170 -> 0.156 ms
    // for the tail).
    const u32 H = cs_log + 1;
    u64 len = L0;
    if constexpr (POL != POL_IP) {
        tail_cluster_rounds<POL, FW>(sm, Ll, len, cs_log, rank, a, w, sh);
        if (rank != 0) return;    // no remote access to this CTA follows
        tail_loop<POL, FW>(sm + Ll / 2, Ll, len, H, true, a, w, sh);
    } else {
        for (u32 k = 0; k < a.nrounds; k++) {
            const bool cl = k < H;             // a cluster round: every CTA
            if (!cl && rank != 0) break;       // the others are done (no remote access to them follows)
            const bool handoff = k + 1 == H;   // the fold goes to CTA 0's rows
            u64* smb = cl ? sm : sm + Ll / 2;  // CTA 0 continues on rows from offset Ll / 2
            const u64 ll = cl ? len >> cs_log : len;   // entries per row this round (>= 4 in cluster rounds)
            const bool active = (u64)warp * 32 < (ll >> 2);
            P acc;
            F3 raw[P::NRAW];
    #pragma unroll
            for (int i = 0; i < P::NRAW; i++) raw[i] = f3_zero();
            if (active) {
                acc.init();
                tail_fold_eval<POL, FW>(smb, Ll, ll, sh.chal, acc, [&](int t, u64 q, u64 Q, const F3& l, const F3& h) {
                    if (!handoff) {
                        sm_st<FW>(smb, Ll, t, q, l);
                        sm_st<FW>(smb, Ll, t, q + Q, h);
                        return;
                    }
                    // the folded table (L0 / 2^H = Ll / 2 entries) goes to CTA
                    // 0's rows from offset Ll / 2 on, at its global index
                    const u64 g_lo = cl_global(q, rank, cs_log), g_hi = cl_global(q + Q, rank, cs_log);
                    u64* row = sm + (u64)(t * FW) * Ll + Ll / 2;
                    dsmem_st(row + g_lo, 0, l.c0);
                    dsmem_st(row + g_hi, 0, h.c0);
                    if (FW == 3) {
                        dsmem_st(row + Ll + g_lo, 0, l.c1);
                        dsmem_st(row + Ll + g_hi, 0, h.c1);
                        dsmem_st(row + 2 * Ll + g_lo, 0, l.c2);
                        dsmem_st(row + 2 * Ll + g_hi, 0, h.c2);
                    }
                });
                acc.result(raw);
            }
            len >>= 1;
            tail_block_reduce<P::NRAW>(raw, active, sh);
            if (cl) {
                if (warp == 0 && lane < NW3) dsmem_st(&sh.cred[rank][lane], 0, sh.tot[lane]);
                cluster_sync_all();   // all CTAs' sums (and after the hand-off the table) are in CTA 0
            }
            if (rank == 0 && warp == 0) {
                if (cl && lane < NW3) {
                    u64 v = 0;
                    for (u32 c = 0; c < CS; c++) v = gl_add(v, sh.cred[c][lane]);
                    sh.tot[lane] = v;
                }
                __syncwarp();
                tail_transcript<POL>(w, a, k, sh);
                __syncwarp();
                if (cl && lane >= 1 && (u32)lane < CS)
                    for (int c = 0; c < 3; c++) dsmem_st(&sh.chal[c], (u32)lane, sh.chal[c]);
            }
            if (cl) cluster_sync_all();   // the challenge is in every CTA
            else __syncthreads();
        }
        if (rank != 0) return;
        tail_finish<POL, FW>(sm + Ll / 2, Ll, len, a, w, sh);
    }
}

template <int POL, int FW>
__global__ void __launch_bounds__(TAIL_TPB, 1) k_tail_one(TailArgs a) {
    chain_enter();
    tail_body<POL, FW>(a);
}
template <int POL, int FW>
__global__ void __launch_bounds__(TAIL_TPB, 1) k_tail_many(const TailArgs* args) { tail_body<POL, FW>(args[blockIdx.x]); }

u64 tail_max_len(int pol, int fw, u64 smem_cap) {
    const u64 per = (u64)pol_ntables(pol) * fw * sizeof(u64);
    u64 L = 1;
    while (2 * L * per <= smem_cap) L *= 2;
    return L;
}

template <int POL, int FW>
static bool tail_inst(const TailArgs* dev_args, const TailArgs* one, u32 n, u64 smem_len, cudaStream_t s) {
    const size_t bytes = (size_t)pol_ntables(POL) * FW * smem_len * sizeof(u64);
    if (bytes > TAIL_SMEM_CAP) return false;
    if (one) {
        cudaFuncSetAttribute(k_tail_one<POL, FW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        return launch_chain(k_tail_one<POL, FW>, 1, TAIL_TPB, bytes, s, *one);
    } else {
        cudaFuncSetAttribute(k_tail_many<POL, FW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        k_tail_many<POL, FW><<<n, TAIL_TPB, bytes, s>>>(dev_args);
    }
    return true;
}

template <int POL, int FW>
static bool tail_cluster_inst(const TailArgs& a, u32 cs_log, cudaStream_t s) {
    const u32 CS = 1u << cs_log;
    const size_t bytes = (size_t)pol_ntables(POL) * FW * (a.L >> cs_log) * sizeof(u64);
    if (bytes > TAIL_SMEM_CAP || CS > (u32)TAIL_MAX_CS) return false;
    cudaFuncSetAttribute(k_tail_cluster<POL, FW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
    if (CS > 8) cudaFuncSetAttribute(k_tail_cluster<POL, FW>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CS, 1, 1);
    cfg.blockDim = dim3(TAIL_TPB, 1, 1);
    cfg.dynamicSmemBytes = bytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_tail_cluster<POL, FW>, a, cs_log) == cudaSuccess;
}

// Largest cluster the device runs for the cluster tail (8 or 16 CTAs of
// TAIL_SMEM_CAP bytes each; 0 when none fits).
u32 tail_cluster_max(void) {
    static std::atomic<int> cached[64];   // per device: 0 unknown, else size + 1
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::atomic<int>& slot = cached[dev & 63];
    int v = slot.load();
    if (v > 0) return (u32)(v - 1);
    v = 0;
    for (u32 cs : {16u, 8u}) {
        cudaFuncSetAttribute(k_tail_cluster<POL_ML, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        if (cs > 8 && cudaFuncSetAttribute(k_tail_cluster<POL_ML, 3>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs, 1, 1);
        cfg.blockDim = dim3(TAIL_TPB, 1, 1);
        cfg.dynamicSmemBytes = TAIL_SMEM_CAP;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_tail_cluster<POL_ML, 3>, &cfg) == cudaSuccess && n > 0) { v = (int)cs; break; }
        cudaGetLastError();
    }
    slot.store(v + 1);
    return (u32)v;
}

bool launch_tail_cluster(int pol, int fw, const TailArgs& a, u32 cs_log, cudaStream_t s) {
    switch (pol * 4 + fw) {
    case POL_ML * 4 + 1: return tail_cluster_inst<POL_ML, 1>(a, cs_log, s);
    case POL_ML * 4 + 3: return tail_cluster_inst<POL_ML, 3>(a, cs_log, s);
    case POL_IP * 4 + 1: return tail_cluster_inst<POL_IP, 1>(a, cs_log, s);
    case POL_IP * 4 + 3: return tail_cluster_inst<POL_IP, 3>(a, cs_log, s);
    default: return false;
    }
}

bool launch_tail(int pol, int fw, const TailArgs* dev_args, const TailArgs* one, u32 n, u64 smem_len, cudaStream_t s) {
    if (!n) return true;
    switch (pol * 4 + fw) {
    case POL_ML * 4 + 1: return tail_inst<POL_ML, 1>(dev_args, one, n, smem_len, s);
    case POL_ML * 4 + 3: return tail_inst<POL_ML, 3>(dev_args, one, n, smem_len, s);
    case POL_IP * 4 + 1: return tail_inst<POL_IP, 1>(dev_args, one, n, smem_len, s);
    case POL_IP * 4 + 3: return tail_inst<POL_IP, 3>(dev_args, one, n, smem_len, s);
    default: return false;
    }
}

}  // namespace effsc
