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
// kernels), reduces across the block, and runs the transcript step
// (finalize_warp: wire values, hook bytes, challenge squeeze).  After the
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

// Shared-memory layout: table t, component c, element i at sm[(t*FW + c)*L0 + i]
// with L0 the starting length (rows keep their stride as the tables shrink).
template <int POL, int FW>
__device__ void tail_body(const TailArgs& a) {
    extern __shared__ __align__(16) u64 sm[];
    __shared__ RoundArgs ra;
    constexpr int NT = Policy<POL, 0>::NT;
    constexpr u32 MF = FW == 3 ? (1u << NT) - 1 : 0;
    constexpr bool E = FW == 3;
    using P = Policy<POL, MF>;
    const u64 L0 = a.L;
    // load (base components of an Fp3-width table read as zero)
    for (int t = 0; t < NT; t++)
        for (int c = 0; c < FW; c++) {
            const u64* src = (c == 0 || ((a.in_ext >> t) & 1u)) ? a.in[t][c] : nullptr;
            u64* dst = sm + (u64)(t * FW + c) * L0;
            for (u64 i = threadIdx.x; i < L0; i += TPB) dst[i] = src ? src[i] : 0;
        }
    if (threadIdx.x == 0) {
        memset(&ra, 0, sizeof ra);
        ra.tx.tx = a.tx;
        ra.tx.hook = a.hook;
        ra.tx.hook_len = a.hook_len;
    }
    __syncthreads();
    const int nwire = pol_nwire_dev(POL);
    u64 len = L0;
    bool fold = a.first_fold != 0;
    F3 ch = fold ? f3_make(a.chal_in[0], a.chal_in[1], a.chal_in[2]) : f3_make(0, 0, 0);
    for (u32 k = 0; k < a.nrounds; k++) {
        if (threadIdx.x == 0) {
            ra.tx.proof_wire = a.proof_wire + (u64)k * 3 * nwire;
            ra.tx.proof_chal = a.proof_chal + (u64)k * 3;
        }
        P acc;
        acc.init();
        F3 lo[NT], hi[NT];
        if (fold) {
            const Mul3 m = mul3_prepare<E>(ch);
            const u64 Q = len >> 2;
            for (u64 q = threadIdx.x; q < Q; q += TPB) {
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
        } else {
            const u64 half = len >> 1;
            if (len == 1) {
                if (threadIdx.x == 0) {
#pragma unroll
                    for (int t = 0; t < NT; t++) lo[t] = sm_ld<FW>(sm, L0, t, 0);
                    acc.single(lo);
                }
            } else {
                for (u64 j = threadIdx.x; j < half; j += TPB) {
#pragma unroll
                    for (int t = 0; t < NT; t++) { lo[t] = sm_ld<FW>(sm, L0, t, j); hi[t] = sm_ld<FW>(sm, L0, t, j + half); }
                    acc.pair(lo, hi);
                }
            }
        }
        F3 raw[P::NRAW];
        acc.result(raw);
        reduce_and_finalize_seg<P::NRAW>(raw, ra, POL, 1, 0);
        __syncthreads();
        const u64* c = a.proof_chal + (u64)k * 3;
        ch = f3_make(c[0], c[1], c[2]);
        fold = true;
    }
    // write back the tables after the last fold
    if (a.out[0][0]) {
        for (int t = 0; t < NT; t++)
            for (int c = 0; c < FW; c++) {
                const u64* src = sm + (u64)(t * FW + c) * L0;
                u64* dst = a.out[t][c];
                for (u64 i = threadIdx.x; i < len; i += TPB) dst[i] = src[i];
            }
    }
}

template <int POL, int FW>
__global__ void __launch_bounds__(TPB) k_tail_one(TailArgs a) { tail_body<POL, FW>(a); }
template <int POL, int FW>
__global__ void __launch_bounds__(TPB) k_tail_many(const TailArgs* args) { tail_body<POL, FW>(args[blockIdx.x]); }

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
        k_tail_one<POL, FW><<<1, TPB, bytes, s>>>(*one);
    } else {
        cudaFuncSetAttribute(k_tail_many<POL, FW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        k_tail_many<POL, FW><<<n, TPB, bytes, s>>>(dev_args);
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
