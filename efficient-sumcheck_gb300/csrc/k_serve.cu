// k_serve.cu -- one launch per serving step: every admitted request advances
// by one round (or finalises), whatever its kind, size and round.
//
// A step's grid is the concatenation of the requests' block ranges; segment k
// (sorted by first block) names its RoundArgs (args[k]) and what the request
// does this step: evaluate round 0 on its base tables, fold + evaluate from
// base or Fp3 tables, the two-pass start of an InnerProduct proof (rounds 0-1,
// then round 2 with the double fold), or the final fold and final value.  The branch is
// uniform per block, so each block runs exactly the single-instance body.
#include "ip01.cuh"

namespace effsc {

__device__ __forceinline__ const ServeSeg& find_seg(const ServeSeg* segs, u32 nsegs, u32& k) {
    __shared__ u32 s_k;
    if (threadIdx.x == 0) {
        u32 lo = 0, hi = nsegs - 1;
        while (lo < hi) {
            u32 mid = (lo + hi + 1) >> 1;
            if (segs[mid].first_block <= blockIdx.x) lo = mid; else hi = mid - 1;
        }
        s_k = lo;
    }
    __syncthreads();
    k = s_k;
    return segs[k];
}

// SumcheckProver::finalize + final_value of an MSB IP / ML prover whose
// tables have length 2 (src/provers/inner_product.rs:115-126,
// src/provers/multilinear.rs:69-79).  `ext`: tables stored with 3 components.
__device__ __forceinline__ void final_body(const RoundArgs& a, int pol, bool ext) {
    if (threadIdx.x != 0) return;
    const F3 rr = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    const Mul3 m = mul3_prepare<true>(rr);
    F3 v[2];
    const int nt = pol == POL_IP ? 2 : 1;
    for (int t = 0; t < nt; t++) {
        F3 lo = ext ? ld<true>(a.t[t].in, 0) : ld<false>(a.t[t].in, 0);
        F3 hi = ext ? ld<true>(a.t[t].in, 1) : ld<false>(a.t[t].in, 1);
        v[t] = f3_fold<true, true>(lo, hi, m);
    }
    const F3 f = nt == 2 ? f3_mul<true, true>(v[0], v[1]) : v[0];
    a.result[0] = f.c0;
    a.result[1] = f.c1;
    a.result[2] = f.c2;
}

template <int POL>
__device__ __forceinline__ void serve_dispatch(const RoundArgs& sa, u32 code, u32 bid, u32 nb) {
    constexpr u32 FULL = POL == POL_IP ? 3u : 1u;
    const bool f3 = code & SERVE_FP3;
    switch (code >> SERVE_PHASE_SHIFT) {
    case SERVE_EVAL: eval_body<POL, SEM_MSB_PAD, 0>(sa, bid, nb); break;
    case SERVE_FOLD_BASE:
        if (f3) fused_body<POL, SEM_MSB_PAD, 0, true>(sa, bid, nb);
        else fused_body<POL, SEM_MSB_PAD, 0, false>(sa, bid, nb);
        break;
    case SERVE_FOLD_EXT: fused_body<POL, SEM_MSB_PAD, FULL, true>(sa, bid, nb); break;
    case SERVE_FINAL_BASE: final_body(sa, POL, false); break;
    case SERVE_FINAL_EXT: final_body(sa, POL, true); break;
    case SERVE_IP01: if (POL == POL_IP) ip01_body<false>(sa, bid, nb); break;
    case SERVE_IP2X: if (POL == POL_IP) ip2x_body<false>(sa, bid, nb); break;
    default: break;
    }
}

__global__ void __launch_bounds__(TPB, 2) k_serve_step(const ServeSeg* segs, u32 nsegs, const RoundArgs* args) {
    __shared__ __align__(16) RoundArgs sa;
    u32 k;
    const ServeSeg sg = find_seg(segs, nsegs, k);
    const u32* src = (const u32*)(args + k);
    u32* dst = (u32*)&sa;
    for (u32 w = threadIdx.x; w < sizeof(RoundArgs) / 4; w += TPB) dst[w] = src[w];
    __syncthreads();
    const u32 bid = blockIdx.x - sg.first_block;
    if (sg.code & SERVE_IP) serve_dispatch<POL_IP>(sa, sg.code, bid, sg.nblocks);
    else serve_dispatch<POL_ML>(sa, sg.code, bid, sg.nblocks);
}

void launch_serve_step(const ServeSeg* segs, u32 nsegs, const RoundArgs* args, u32 grid, cudaStream_t s) {
    if (!nsegs || !grid) return;
    k_serve_step<<<grid, TPB, 0, s>>>(segs, nsegs, args);
}

}  // namespace effsc
