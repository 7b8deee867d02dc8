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

// Shared-memory layout: table t, component c, element i at sm[(t*FW + c)*L0 + i]
// with L0 the starting length (rows keep their stride as the tables shrink).
// Warp 0 keeps the transcript state in registers for the whole tail and the
// challenge stays in shared memory, so a round costs one block reduction and
// one transcript step.
template <int POL, int FW>
__device__ void tail_body(const TailArgs& a) {
    extern __shared__ __align__(16) u64 sm[];
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 MF = FW == 3 ? (1u << NT) - 1 : 0;
    constexpr bool E = FW == 3;
    using P = Policy<POL, MF>;
    constexpr int NW3 = 3 * P::NRAW;
    // ML and IP send their raw sums as the wire values: [s0] / [q0, qinf]
    constexpr int NWIRE = POL == POL_ML ? 1 : 2;
    __shared__ u64 s_red[TAIL_NW][NW3];
    __shared__ u64 s_tot[NW3];
    __shared__ u64 s_chal[3];
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 L0 = a.L;
    for (int t = 0; t < NT; t++)
        for (int c = 0; c < FW; c++) {
            const u64* src = (c == 0 || ((a.in_ext >> t) & 1u)) ? a.in[t][c] : nullptr;
            u64* dst = sm + (u64)(t * FW + c) * L0;
            for (u64 i = threadIdx.x; i < L0; i += TAIL_TPB) dst[i] = src ? src[i] : 0;
        }
    if (threadIdx.x < 3) s_chal[threadIdx.x] = a.first_fold ? a.chal_in[threadIdx.x] : 0;
    DevTranscript* T = (DevTranscript*)a.tx;
    WarpTx w;
    if (warp == 0) w = tx_load(T, lane);
    __syncthreads();
    u64 len = L0;
    bool fold = a.first_fold != 0;
    for (u32 k = 0; k < a.nrounds; k++) {
        // warps without entries this round skip the arithmetic and the
        // reduction of their (zero) sums; every warp reaches both barriers
        const u64 nwork = fold ? (len >> 2) : len == 1 ? 1 : (len >> 1);
        const bool active = (u64)warp * 32 < nwork;
        P acc;
        F3 raw[P::NRAW];
#pragma unroll
        for (int i = 0; i < P::NRAW; i++) raw[i] = f3_zero();
        if (fold && !active) len >>= 1;
        if (active) {
            acc.init();
            F3 lo[NT], hi[NT];
            if (fold) {
                const Mul3 m = mul3_prepare<E>(f3_make(s_chal[0], s_chal[1], s_chal[2]));
                const u64 Q = len >> 2;
                for (u64 q = threadIdx.x; q < Q; q += TAIL_TPB) {
#pragma unroll
                    for (int t = 0; t < NT; t++) {
                        F3 x0 = sm_ld<FW>(sm, L0, t, q), x1 = sm_ld<FW>(sm, L0, t, q + Q);
                        F3 x2 = sm_ld<FW>(sm, L0, t, q + 2 * Q), x3 = sm_ld<FW>(sm, L0, t, q + 3 * Q);
                        lo[t] = f3_fold<E, E>(x0, x2, m);
                        hi[t] = f3_fold<E, E>(x1, x3, m);
                        sm_st<FW>(sm, L0, t, q, lo[t]);
                        sm_st<FW>(sm, L0, t, q + Q, hi[t]);
                    }
                    acc.pair(lo, hi);
                }
                len >>= 1;
            } else if (len == 1) {
                if (threadIdx.x == 0) {
#pragma unroll
                    for (int t = 0; t < NT; t++) lo[t] = sm_ld<FW>(sm, L0, t, 0);
                    acc.single(lo);
                }
            } else {
                const u64 half = len >> 1;
                for (u64 j = threadIdx.x; j < half; j += TAIL_TPB) {
#pragma unroll
                    for (int t = 0; t < NT; t++) { lo[t] = sm_ld<FW>(sm, L0, t, j); hi[t] = sm_ld<FW>(sm, L0, t, j + half); }
                    acc.pair(lo, hi);
                }
            }
            acc.result(raw);
            // block reduction
#pragma unroll
            for (int off = 16; off; off >>= 1) {
#pragma unroll
                for (int i = 0; i < P::NRAW; i++) {
                    raw[i].c0 = gl_add(raw[i].c0, __shfl_down_sync(0xffffffffu, raw[i].c0, off));
                    raw[i].c1 = gl_add(raw[i].c1, __shfl_down_sync(0xffffffffu, raw[i].c1, off));
                    raw[i].c2 = gl_add(raw[i].c2, __shfl_down_sync(0xffffffffu, raw[i].c2, off));
                }
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < P::NRAW; i++) { s_red[warp][3 * i] = raw[i].c0; s_red[warp][3 * i + 1] = raw[i].c1; s_red[warp][3 * i + 2] = raw[i].c2; }
        }
        __syncthreads();
        if (warp == 0) {
            if (lane < NW3) {
                u64 v = 0;
#pragma unroll
                for (int q = 0; q < TAIL_NW; q++) v = gl_add(v, s_red[q][lane]);
                s_tot[lane] = v;
            }
            __syncwarp();
            // transcript step (src/runner.rs:39-55)
            tx_send_elems(w, lane, s_tot, NWIRE);
            if (a.hook_len) {
                const uint8_t* hk = a.hook;
                if (((w.pos & 7) == 0 || w.squeezing) && (a.hook_len & 7) == 0 && ((uintptr_t)hk & 7) == 0) {
                    const u64* hw = (const u64*)hk;
                    tx_absorb_words(w, lane, a.hook_len >> 3, [&](u32 i) -> u64 { return hw[i]; });
                } else {
                    tx_absorb(w, lane, a.hook_len, [&](u32 i) -> uint8_t { return hk[i]; });
                }
            }
            tx_challenge(w, lane, s_chal, s_scr);
            if (lane < 3 * NWIRE) a.proof_wire[(u64)k * 3 * NWIRE + lane] = s_tot[lane];
            if (lane < 3) a.proof_chal[(u64)k * 3 + lane] = s_chal[lane];
        }
        __syncthreads();
        fold = true;
    }
    if (warp == 0) tx_store(T, w, lane);
    // write back the tables after the last fold
    if (a.out[0][0]) {
        for (int t = 0; t < NT; t++)
            for (int c = 0; c < FW; c++) {
                const u64* src = sm + (u64)(t * FW + c) * L0;
                u64* dst = a.out[t][c];
                for (u64 i = threadIdx.x; i < len; i += TAIL_TPB) dst[i] = src[i];
            }
    }
}

template <int POL, int FW>
__global__ void __launch_bounds__(TAIL_TPB, 1) k_tail_one(TailArgs a) { tail_body<POL, FW>(a); }
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
        k_tail_one<POL, FW><<<1, TAIL_TPB, bytes, s>>>(*one);
    } else {
        cudaFuncSetAttribute(k_tail_many<POL, FW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        k_tail_many<POL, FW><<<n, TAIL_TPB, bytes, s>>>(dev_args);
    }
    return true;
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
