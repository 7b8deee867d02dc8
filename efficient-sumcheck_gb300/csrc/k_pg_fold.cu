// k_pg_fold.cu -- protogalaxy::fold (src/folding.rs:14-75) on the device.
//
// n = 2^K polynomials of w coefficients are folded pairwise, level by level:
//   out_i(X) = p_2i(X) + (a + b X) (p_2i+1(X) - p_2i(X)),
// i.e. coefficient j of out_i is p0[j] + a d[j] + b d[j-1] with d = p1 - p0
// (d[-1] = d[w] = 0); each level adds one coefficient.  One pass folds g
// levels of a group of 2^g consecutive polynomials inside shared memory (the
// group is a contiguous block of the input, read once, coalesced), so the
// input is read from HBM once and the pass writes 2^-g of it; two or three
// passes finish any size.  Polynomials too wide for a shared-memory group
// use a per-level kernel on global memory.
//
// Element layout: AoS, `field` 64-bit words per coefficient (Fp: 1, Fp3: 3),
// ascending degree, rows of `width` coefficients.  Both fields run the same
// code with E = (field == 3); the sum a d[j] + b d[j-1] + p0[j] is accumulated
// lazily (160-bit accumulators) and reduced once per output word.
#include "effsc_gpu.h"
#include "kernels.h"
#include "round_common.cuh"

#include <algorithm>
#include <vector>

using namespace effsc;

int effsc_internal_ctx_device(const effsc_ctx* c);
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c);
uint64_t effsc_internal_add_launches(uint64_t k);
const u64* effsc_internal_device_view(int device, const uint64_t* ptr, bool* is_host);

namespace effsc {

constexpr int PG_TPB = 256;
constexpr size_t PG_SMEM = 48 * 1024;   // per block: four blocks per SM
constexpr u32 PG_MAX_G = 10;

template <bool E>
__device__ __forceinline__ F3 pg_load(const u64* p, size_t e) {
    return E ? f3_make(p[3 * e], p[3 * e + 1], p[3 * e + 2]) : f3_make(p[e], 0, 0);
}
template <bool E>
__device__ __forceinline__ void pg_store(u64* p, size_t e, const F3& v) {
    if (E) { p[3 * e] = v.c0; p[3 * e + 1] = v.c1; p[3 * e + 2] = v.c2; }
    else p[e] = v.c0;
}
// x * m accumulated into (s0, s1, s2) without reduction.
template <bool E>
__device__ __forceinline__ void pg_mac(Acc& s0, Acc& s1, Acc& s2, const F3& x, const Mul3& m) {
    acc_mac(s0, x.c0, m.m0);
    if (E) {
        acc_mac(s0, x.c1, m.w2); acc_mac(s0, x.c2, m.w1);
        acc_mac(s1, x.c0, m.m1); acc_mac(s1, x.c1, m.m0); acc_mac(s1, x.c2, m.w2);
        acc_mac(s2, x.c0, m.m2); acc_mac(s2, x.c1, m.m1); acc_mac(s2, x.c2, m.m0);
    }
}
// p0 + a d + b dm1
template <bool E>
__device__ __forceinline__ F3 pg_coef(const F3& p0, const F3& d, const F3& dm1, const Mul3& a, const Mul3& b) {
    Acc s0 = acc_from(p0.c0), s1 = acc_from(E ? p0.c1 : 0), s2 = acc_from(E ? p0.c2 : 0);
    pg_mac<E>(s0, s1, s2, d, a);
    pg_mac<E>(s0, s1, s2, dm1, b);
    F3 r;
    r.c0 = acc_reduce(s0);
    if (E) { r.c1 = acc_reduce(s1); r.c2 = acc_reduce(s2); } else { r.c1 = r.c2 = 0; }
    return r;
}

// One block folds g levels of 2^g consecutive rows of width w.  Shared
// memory: A (2^g rows) and B (2^(g-1) rows), row stride w + g coefficients.
template <bool E>
__global__ void __launch_bounds__(PG_TPB) k_pg_group(const u64* __restrict__ in, u32 w, u32 g,
                                                     const u64* __restrict__ pairs, u64* __restrict__ out) {
    extern __shared__ u64 sm[];
    constexpr u32 EW = E ? 3 : 1;
    const u32 S = w + g, R = 1u << g;
    u64* A = sm;
    u64* B = sm + (size_t)R * S * EW;
    const u32 row_words = w * EW;
    const u64* src = in + (size_t)blockIdx.x * R * row_words;
    for (u32 t = threadIdx.x; t < R * row_words; t += PG_TPB) {
        const u32 row = t / row_words, rem = t - row * row_words;
        A[row * S * EW + rem] = src[t];
    }
    __syncthreads();
    for (u32 l = 0; l < g; l++) {
        const u64* s = (l & 1) ? B : A;
        u64* d = (l & 1) ? A : B;
        const u32 cnt = R >> (l + 1), wl = w + l, wo = wl + 1;
        const Mul3 ma = mul3_prepare<E>(f3_make(pairs[6 * l], pairs[6 * l + 1], pairs[6 * l + 2]));
        const Mul3 mb = mul3_prepare<E>(f3_make(pairs[6 * l + 3], pairs[6 * l + 4], pairs[6 * l + 5]));
        for (u32 idx = threadIdx.x; idx < cnt * wo; idx += PG_TPB) {
            const u32 i = idx / wo, j = idx - i * wo;
            const u64* p0 = s + (size_t)(2 * i) * S * EW;
            const u64* p1 = p0 + (size_t)S * EW;
            const F3 z = f3_zero();
            const F3 b0 = j < wl ? pg_load<E>(p0, j) : z;
            const F3 dj = j < wl ? f3_sub<E>(pg_load<E>(p1, j), b0) : z;
            const F3 dm = j > 0 ? f3_sub<E>(pg_load<E>(p1, j - 1), pg_load<E>(p0, j - 1)) : z;
            pg_store<E>(d + (size_t)i * S * EW, j, pg_coef<E>(b0, dj, dm, ma, mb));
        }
        __syncthreads();
    }
    const u64* res = (g & 1) ? B : A;
    u64* dst = out + (size_t)blockIdx.x * S * EW;
    for (u32 t = threadIdx.x; t < S * EW; t += PG_TPB) dst[t] = res[t];
}

// One level on global memory: cnt output rows of width w + 1 from 2 cnt
// input rows of width w.
template <bool E>
__global__ void __launch_bounds__(PG_TPB) k_pg_level(const u64* __restrict__ in, size_t cnt, u32 w,
                                                     const u64* __restrict__ pair, u64* __restrict__ out) {
    const Mul3 ma = mul3_prepare<E>(f3_make(pair[0], pair[1], pair[2]));
    const Mul3 mb = mul3_prepare<E>(f3_make(pair[3], pair[4], pair[5]));
    const u32 wo = w + 1;
    for (size_t idx = (size_t)blockIdx.x * PG_TPB + threadIdx.x; idx < cnt * wo; idx += (size_t)gridDim.x * PG_TPB) {
        const size_t i = idx / wo;
        const u32 j = (u32)(idx - i * wo);
        const u64* p0 = in + 2 * i * w * (E ? 3 : 1);
        const u64* p1 = p0 + (size_t)w * (E ? 3 : 1);
        const F3 z = f3_zero();
        const F3 b0 = j < w ? pg_load<E>(p0, j) : z;
        const F3 dj = j < w ? f3_sub<E>(pg_load<E>(p1, j), b0) : z;
        const F3 dm = j > 0 ? f3_sub<E>(pg_load<E>(p1, j - 1), pg_load<E>(p0, j - 1)) : z;
        pg_store<E>(out + i * wo * (E ? 3 : 1), j, pg_coef<E>(b0, dj, dm, ma, mb));
    }
}

size_t pg_group_smem(u32 w, u32 g, u32 ew) { return (size_t)3 * (1u << (g - 1)) * (w + g) * ew * 8; }

// Levels one shared-memory pass folds for `count` rows of width w (0: none fit).
u32 pg_plan_levels(size_t count, u32 w, u32 ew) {
    u32 g = 0;
    while (g < PG_MAX_G && ((size_t)2 << g) <= count && pg_group_smem(w, g + 1, ew) <= PG_SMEM) g++;
    return g;
}

}  // namespace effsc

#define PCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) { rc = effsc_set_error(EFFSC_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); goto done; } \
    } while (0)

extern "C" int effsc_protogalaxy_fold(effsc_ctx* ctx, int field, const uint64_t* pairs, size_t n_levels,
                                      const uint64_t* polys, size_t n_polys, size_t width, uint64_t* out,
                                      size_t* out_len) {
    if (!ctx || !out_len || (n_levels && !pairs) || (n_polys && width && !polys) || (n_polys && !out))
        return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    if (field != EFFSC_FP && field != EFFSC_FP3) return effsc_set_error(EFFSC_INVALID_ARG, "bad field");
    if (width > (1u << 20) || n_levels > 64) return effsc_set_error(EFFSC_INVALID_ARG, "width or levels too large");
    if (n_polys / 2 > 0x7FFFFFFFull) return effsc_set_error(EFFSC_UNSUPPORTED, "more than 2^32 polynomials");
    const u32 ew = (u32)field;
    *out_len = 0;
    if (n_polys == 0) return EFFSC_OK;
    const int dev = effsc_internal_ctx_device(ctx);
    cudaStream_t s = effsc_internal_ctx_stream(ctx);
    if (cudaSetDevice(dev) != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "cudaSetDevice");
    // levels that run: a release build stops changing the result once one
    // polynomial is left, and drops an odd last one at each level
    u32 K = 0;
    if (n_polys >= 2)
        while (K < n_levels && ((size_t)2 << K) <= n_polys) K++;
    const size_t count0 = (size_t)1 << K;
    const size_t final_w = width + K;
    std::vector<u64> res(std::max<size_t>(final_w, 1) * ew, 0), pr(std::max<size_t>(K, 1) * 6, 0);
    for (u32 k = 0; k < K; k++)
        for (int h = 0; h < 2; h++)
            for (u32 c = 0; c < ew; c++) pr[6 * k + 3 * h + c] = pairs[(2 * k + h) * ew + c] % 0xFFFFFFFF00000001ULL;
    int rc = EFFSC_OK;
    u64 *d_pairs = nullptr, *d_in = nullptr, *bufs[2] = {nullptr, nullptr};
    const u64* cur = nullptr;
    if (width) {
        bool is_host = false;
        cur = effsc_internal_device_view(dev, polys, &is_host);
        if (!cur) {
            const size_t bytes = count0 * width * ew * 8;
            PCK(cudaMallocAsync((void**)&d_in, bytes, s));
            PCK(cudaMemcpyAsync(d_in, polys, bytes, cudaMemcpyHostToDevice, s));
            cur = d_in;
        }
    }
    if (K && width) {
        PCK(cudaMallocAsync((void**)&d_pairs, pr.size() * 8, s));
        PCK(cudaMemcpyAsync(d_pairs, pr.data(), pr.size() * 8, cudaMemcpyHostToDevice, s));
        size_t count = count0;
        u32 w = (u32)width, lvl = 0;
        int which = 0;
        size_t cap[2] = {0, 0};
        while (count > 1) {
            u32 g = pg_plan_levels(count, w, ew);
            const size_t out_rows = g ? count >> g : count >> 1;
            const u32 out_w = w + (g ? g : 1);
            const size_t need = out_rows * out_w * ew * 8;
            if (need > cap[which]) {
                if (bufs[which]) cudaFreeAsync(bufs[which], s);
                bufs[which] = nullptr;
                cap[which] = 0;
                PCK(cudaMallocAsync((void**)&bufs[which], need, s));
                cap[which] = need;
            }
            if (g) {
                const size_t smem = pg_group_smem(w, g, ew);
                if (ew == 3) k_pg_group<true><<<(unsigned)out_rows, PG_TPB, smem, s>>>(cur, w, g, d_pairs + 6 * lvl, bufs[which]);
                else k_pg_group<false><<<(unsigned)out_rows, PG_TPB, smem, s>>>(cur, w, g, d_pairs + 6 * lvl, bufs[which]);
                lvl += g;
            } else {
                const size_t items = out_rows * (w + 1);
                const unsigned grid = (unsigned)std::min<size_t>((items + PG_TPB - 1) / PG_TPB, 152 * 16);
                if (ew == 3) k_pg_level<true><<<grid, PG_TPB, 0, s>>>(cur, out_rows, w, d_pairs + 6 * lvl, bufs[which]);
                else k_pg_level<false><<<grid, PG_TPB, 0, s>>>(cur, out_rows, w, d_pairs + 6 * lvl, bufs[which]);
                lvl += 1;
            }
            effsc_internal_add_launches(1);
            PCK(cudaGetLastError());
            cur = bufs[which];
            which ^= 1;
            count = out_rows;
            w = out_w;
        }
    }
    if (final_w && width) PCK(cudaMemcpyAsync(res.data(), cur, final_w * ew * 8, cudaMemcpyDefault, s));
    PCK(cudaStreamSynchronize(s));
    {
        size_t len = final_w;
        auto zero = [&](size_t e) {
            for (u32 c = 0; c < ew; c++)
                if (res[e * ew + c]) return false;
            return true;
        };
        const size_t keep = n_polys >= 2 ? 1 : 0;    // to_dense_poly keeps one term; a lone input is returned as is
        while (len > keep && zero(len - 1)) len--;
        if (n_polys >= 2 && len == 0) len = 1;       // width 0: the zero polynomial as one term
        for (size_t e = 0; e < len; e++)
            for (u32 c = 0; c < ew; c++) out[e * ew + c] = e < final_w ? res[e * ew + c] : 0;
        *out_len = len;
    }
done:
    for (void* p : {(void*)d_pairs, (void*)d_in, (void*)bufs[0], (void*)bufs[1]})
        if (p) cudaFreeAsync(p, s);
    return rc;
}
