// k_batch.cu -- the final folds of a batch of independent provers in one
// launch (the batch's round steps run k_serve_step, k_serve.cu).
#include "round_common.cuh"

namespace effsc {

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

void launch_batch_finalize(const RoundArgs* args, const unsigned char* ext, u32 n, int ntab, u64* finals, cudaStream_t s) {
    if (!n) return;
    k_batch_finalize<<<(n + 127) / 128, 128, 0, s>>>(args, ext, n, ntab, finals);
}

}  // namespace effsc
