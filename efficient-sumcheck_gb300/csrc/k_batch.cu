// k_batch.cu -- one launch per round for a cohort of independent provers.
//
// A round's grid is the concatenation of every active instance's blocks; the
// segment table (one entry per instance, sorted by first block) maps a block
// to its instance and its index inside that instance's range.  The block
// copies the instance's RoundArgs into shared memory and runs the same
// eval / fused bodies as the single-instance kernels, so each instance gets
// its own grid reduction, wire values and transcript step.
#include "round_common.cuh"

namespace effsc {

__device__ __forceinline__ void load_segment(const BatchSeg* segs, u32 nsegs, const RoundArgs* args,
                                             RoundArgs& sa, u32& bid, u32& nb) {
    __shared__ u32 s_seg;
    if (threadIdx.x == 0) {
        u32 lo = 0, hi = nsegs - 1;
        while (lo < hi) {
            u32 mid = (lo + hi + 1) >> 1;
            if (segs[mid].first_block <= blockIdx.x) lo = mid; else hi = mid - 1;
        }
        s_seg = lo;
    }
    __syncthreads();
    const BatchSeg sg = segs[s_seg];
    const u32* src = (const u32*)(args + sg.inst);
    u32* dst = (u32*)&sa;
    for (u32 w = threadIdx.x; w < sizeof(RoundArgs) / 4; w += TPB) dst[w] = src[w];
    bid = blockIdx.x - sg.first_block;
    nb = sg.nblocks;
    __syncthreads();
}

template <int POL, bool FUSED, u32 M, bool ECH>
__global__ void __launch_bounds__(TPB, 2) k_batch_round(const BatchSeg* segs, u32 nsegs, const RoundArgs* args) {
    __shared__ __align__(16) RoundArgs sa;
    u32 bid, nb;
    load_segment(segs, nsegs, args, sa, bid, nb);
    if (FUSED) fused_body<POL, SEM_MSB_PAD, M, ECH>(sa, bid, nb);
    else eval_body<POL, SEM_MSB_PAD, M>(sa, bid, nb);
}

// Final fold (length 2 -> 1) of every instance and its final value:
// IP: a(r) * b(r) (src/provers/inner_product.rs:115-126); ML: v(r)
// (src/provers/multilinear.rs:69-79).  One thread per instance; ext[i] says
// whether instance i's tables are Fp3 at this point (base values are the
// embedded triples, so the Fp3 formulas apply to both).
__global__ void k_batch_finalize(const RoundArgs* args, const unsigned char* ext, u32 n, int ntab, u64* finals) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const RoundArgs& a = args[i];
    const F3 rr = f3_make(a.chal_ptr[0], a.chal_ptr[1], a.chal_ptr[2]);
    const Mul3 m = mul3_prepare<true>(rr);
    F3 v[2];
    for (int t = 0; t < ntab; t++) {
        F3 lo, hi;
        if (ext[i]) { lo = ld<true>(a.t[t].in, 0); hi = ld<true>(a.t[t].in, 1); }
        else { lo = ld<false>(a.t[t].in, 0); hi = ld<false>(a.t[t].in, 1); }
        v[t] = f3_fold<true, true>(lo, hi, m);
    }
    F3 f = ntab == 2 ? f3_mul<true, true>(v[0], v[1]) : v[0];
    finals[3 * i] = f.c0;
    finals[3 * i + 1] = f.c1;
    finals[3 * i + 2] = f.c2;
}

#define BATCH(POL, FUSED, M, ECH) \
    case ((POL) * 64 + (FUSED) * 32 + (M) * 2 + (ECH)): \
        k_batch_round<POL, FUSED, M, ECH><<<grid, TPB, 0, s>>>(segs, nsegs, args); return true;

bool launch_batch_round(int pol, bool fused, u32 mask, bool ech, const BatchSeg* segs, u32 nsegs,
                        const RoundArgs* args, u32 grid, cudaStream_t s) {
    switch (pol * 64 + (fused ? 32 : 0) + (int)mask * 2 + (ech ? 1 : 0)) {
        BATCH(POL_IP, false, 0, false) BATCH(POL_IP, true, 0, false) BATCH(POL_IP, true, 0, true) BATCH(POL_IP, true, 3, true)
        BATCH(POL_ML, false, 0, false) BATCH(POL_ML, true, 0, false) BATCH(POL_ML, true, 0, true) BATCH(POL_ML, true, 1, true)
        default: return false;
    }
}
void launch_batch_finalize(const RoundArgs* args, const unsigned char* ext, u32 n, int ntab, u64* finals, cudaStream_t s) {
    if (!n) return;
    k_batch_finalize<<<(n + 127) / 128, 128, 0, s>>>(args, ext, n, ntab, finals);
}

}  // namespace effsc
