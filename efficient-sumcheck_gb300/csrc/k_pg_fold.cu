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
#include <atomic>
#include <vector>

using namespace effsc;

int effsc_internal_ctx_device(const effsc_ctx* c);
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c);
uint64_t effsc_internal_add_launches(uint64_t k);
const u64* effsc_internal_device_view(int device, const uint64_t* ptr, bool* is_host);
void* effsc_internal_pinned_get(effsc_ctx* c, size_t bytes);
void effsc_internal_pinned_put(effsc_ctx* c, void* p, size_t bytes);

namespace effsc {

constexpr int PG_TPB = 256;
constexpr size_t PG_SMEM = 48 * 1024;        // wide grids: four blocks per SM
constexpr size_t PG_SMEM_BIG = 200 * 1024;   // narrow grids: fewer passes
constexpr u32 PG_MAX_G = 10;

// The (a, b) multipliers of the levels one pass folds, prepared on the host
// as (m0, m1, m2, W m1, W m2) each and passed by value (no upload).
struct PgMul {
    u64 q[PG_MAX_G * 10];
};

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

template <bool E>
__device__ __forceinline__ Mul3 pg_mul3(const u64* q) {
    Mul3 m;
    m.m0 = q[0];
    m.m1 = E ? q[1] : 0;
    m.m2 = E ? q[2] : 0;
    m.w1 = E ? q[3] : 0;
    m.w2 = E ? q[4] : 0;
    return m;
}

// One block folds g levels of R = 2^g consecutive rows of width w.
// Shared-memory layout: rows are kept as pairs, pair k of a level at k * P
// (P = 2 S + 1 coefficients, S >= w + g the widest row), its first row at
// +0 and its second at +S; the odd pair stride spreads the rows that
// neighbouring threads read over all banks.  Buffer A holds the R rows of
// level 0 (R/2 pairs), B the R/2 rows of level 1; the levels then alternate.
// The group arrives by 8-byte asynchronous copies (cp.async, no register
// staging).  Each level gives every row pair TPB/cnt threads (or every
// thread whole pairs when cnt >= TPB), each computing a run of consecutive
// coefficients, so d[j-1] carries over in a register.
__device__ __forceinline__ void pg_cp8(u64* dst, const u64* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

template <bool E>
__global__ void __launch_bounds__(PG_TPB) k_pg_group(const u64* __restrict__ in, u32 w, u32 g, u32 S,
                                                     const PgMul mul, u64* __restrict__ out) {
    extern __shared__ u64 sm[];
    constexpr u32 EW = E ? 3 : 1;
    const u64* pairs = mul.q;
    const u32 R = 1u << g, P = 2 * S + 1;
    u64* A = sm;
    u64* B = sm + (size_t)(R / 2) * P * EW;
    const u32 row_words = w * EW, total = R * row_words;
    const u64* src = in + (size_t)blockIdx.x * total;
    {
        u32 row = threadIdx.x / row_words, col = threadIdx.x - row * row_words;
        const u32 step_r = PG_TPB / row_words, step_c = PG_TPB - step_r * row_words;
        for (u32 t = threadIdx.x; t < total; t += PG_TPB) {
            pg_cp8(A + ((row >> 1) * P + (row & 1) * S) * EW + col, src + t);
            row += step_r;
            col += step_c;
            if (col >= row_words) { col -= row_words; row++; }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    }
    __syncthreads();
    for (u32 l = 0; l < g; l++) {
        const u64* s = (l & 1) ? B : A;
        u64* d = (l & 1) ? A : B;
        const u32 lg_cnt = g - l - 1, cnt = 1u << lg_cnt, wl = w + l, wo = wl + 1;
        const Mul3 ma = pg_mul3<E>(pairs + 10 * l), mb = pg_mul3<E>(pairs + 10 * l + 5);
        // threads per pair (a power of two) and the run each computes
        const u32 lg_tpp = cnt >= PG_TPB ? 0 : __ffs(PG_TPB) - 1 - lg_cnt;
        const u32 tpp = 1u << lg_tpp, run = (wo + tpp - 1) >> lg_tpp;
        const u32 part = threadIdx.x & (tpp - 1);
        const u32 j0 = part * run, j1 = min(j0 + run, wo);
        for (u32 i = threadIdx.x >> lg_tpp; i < cnt; i += PG_TPB >> lg_tpp) {
            if (j0 >= j1) break;
            const u64* p0 = s + (size_t)i * P * EW;
            const u64* p1 = p0 + (size_t)S * EW;
            u64* o = d + ((size_t)(i >> 1) * P + (i & 1) * S) * EW;
            F3 dm = j0 ? f3_sub<E>(pg_load<E>(p1, j0 - 1), pg_load<E>(p0, j0 - 1)) : f3_zero();
            for (u32 j = j0; j < j1; j++) {
                F3 x0 = f3_zero(), dj = f3_zero();
                if (j < wl) {
                    x0 = pg_load<E>(p0, j);
                    dj = f3_sub<E>(pg_load<E>(p1, j), x0);
                }
                pg_store<E>(o, j, pg_coef<E>(x0, dj, dm, ma, mb));
                dm = dj;
            }
        }
        __syncthreads();
    }
    const u64* res = (g & 1) ? B : A;
    u64* dst = out + (size_t)blockIdx.x * (w + g) * EW;
    for (u32 t = threadIdx.x; t < (w + g) * EW; t += PG_TPB) dst[t] = res[t];
}

// Warp subtrees for the wide first passes: each warp folds gw levels of its
// own R = 2^gw consecutive rows with no block barrier.  Rows are dense in
// shared memory (row i of a level at i * width), and a level's outputs are
// spread over the 32 lanes in order (output k = coefficient k mod wo of row
// k / wo), so every lane has work until the last levels and neighbouring
// lanes read neighbouring words.  Per warp: A holds the R input rows, B the
// R/2 rows of level 1; the levels then alternate.
template <bool E>
__global__ void __launch_bounds__(PG_TPB) k_pg_warp(const u64* __restrict__ in, size_t trees, u32 w, u32 gw,
                                                    const PgMul mul, u64* __restrict__ out) {
    extern __shared__ u64 sm[];
    constexpr u32 EW = E ? 3 : 1;
    const u64* pairs = mul.q;
    const u32 lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t tree = (size_t)blockIdx.x * (PG_TPB / 32) + wid;
    if (tree >= trees) return;
    const u32 R = 1u << gw, a_words = R * w * EW, b_words = (R / 2) * (w + 1) * EW;
    u64* A = sm + (size_t)wid * (a_words + b_words);
    u64* B = A + a_words;
    const u64* src = in + tree * a_words;
    for (u32 t = lane; t < a_words; t += 32) pg_cp8(A + t, src + t);
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
    u32 wl = w;
    for (u32 l = 0; l < gw; l++) {
        const u64* s = (l & 1) ? B : A;
        u64* d = (l & 1) ? A : B;
        const u32 wo = wl + 1, total = (R >> (l + 1)) * wo, pair_words = 2 * wl * EW;
        const Mul3 ma = pg_mul3<E>(pairs + 10 * l), mb = pg_mul3<E>(pairs + 10 * l + 5);
        // lane -> (row pair, coefficient) and the step of 32 outputs, by
        // subtraction (wo >= 2, so at most 16 rounds)
        u32 q32 = 0, r32 = 32, i = 0, j = lane;
        while (r32 >= wo) { r32 -= wo; q32++; }
        while (j >= wo) { j -= wo; i++; }
        u32 row = i * pair_words;                 // word offset of the pair's first row
        const u32 row_step = q32 * pair_words;
        for (u32 k = lane; k < total; k += 32) {
            const u64* p0 = s + row;
            const u64* p1 = p0 + wl * EW;
            F3 x0 = f3_zero(), dj = f3_zero(), dm = f3_zero();
            if (j < wl) {
                x0 = pg_load<E>(p0, j);
                dj = f3_sub<E>(pg_load<E>(p1, j), x0);
            }
            if (j) dm = f3_sub<E>(pg_load<E>(p1, j - 1), pg_load<E>(p0, j - 1));
            pg_store<E>(d, k, pg_coef<E>(x0, dj, dm, ma, mb));
            row += row_step;
            j += r32;
            if (j >= wo) { j -= wo; row += pair_words; }
        }
        __syncwarp();
        wl = wo;
    }
    const u64* res = (gw & 1) ? B : A;
    u64* dst = out + tree * (size_t)wl * EW;
    for (u32 t = lane; t < wl * EW; t += 32) dst[t] = res[t];
}

// One level on global memory: cnt output rows of width w + 1 from 2 cnt
// input rows of width w.
template <bool E>
__global__ void __launch_bounds__(PG_TPB) k_pg_level(const u64* __restrict__ in, size_t cnt, u32 w,
                                                     const PgMul mul, u64* __restrict__ out) {
    const u64* pair = mul.q;
    const Mul3 ma = pg_mul3<E>(pair), mb = pg_mul3<E>(pair + 5);
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

constexpr u64 PG_P = 0xFFFFFFFF00000001ULL;
inline u64 pg_hmul(u64 a, u64 b) { return (u64)(((unsigned __int128)a * b) % PG_P); }

size_t pg_warp_smem(u32 w, u32 gw, u32 ew) {
    const size_t R = (size_t)1 << gw;
    return (R * w + (R / 2) * (w + 1)) * ew * 8;
}
constexpr size_t PG_WARP_SMEM = 12 * 1024;   // per warp
constexpr u32 PG_WARP_MAX_G = 6;
// Levels a warp-subtree pass folds: at least 3 (or all that are left),
// else 0 and the block kernel takes the pass.
u32 pg_plan_warp(size_t count, u32 w, u32 ew) {
    u32 g = 0;
    while (g < PG_WARP_MAX_G && ((size_t)2 << g) <= count && pg_warp_smem(w, g + 1, ew) <= PG_WARP_SMEM) g++;
    return (g >= 3 || (g && (count >> g) == 1)) ? g : 0;
}

// Row width bound of a group (odd, so that the pair stride 2 S + 1 is odd
// as well as the row offset S within a pair).
u32 pg_stride(u32 w, u32 g) { return (w + g) | 1u; }
size_t pg_group_smem(u32 w, u32 g, u32 ew) {
    const size_t R = (size_t)1 << g, pairs_a = R / 2, pairs_b = R >= 4 ? R / 4 : 1;
    return (pairs_a + pairs_b) * (2 * pg_stride(w, g) + 1) * ew * 8;
}

// Levels one shared-memory pass folds for `count` rows of width w (0: none
// fit in `budget` bytes).
u32 pg_plan_levels(size_t count, u32 w, u32 ew, size_t budget) {
    u32 g = 0;
    while (g < PG_MAX_G && ((size_t)2 << g) <= count && pg_group_smem(w, g + 1, ew) <= budget) g++;
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
    // (a, b) per level as prepared multipliers (m0, m1, m2, W m1, W m2)
    std::vector<u64> pr(std::max<size_t>(K, 1) * 10, 0);
    for (u32 k = 0; k < K; k++)
        for (int h = 0; h < 2; h++) {
            u64* q = &pr[10 * k + 5 * h];
            for (u32 c = 0; c < ew; c++) q[c] = pairs[(2 * k + h) * ew + c] % PG_P;
            q[3] = pg_hmul(GL_W, q[1]);
            q[4] = pg_hmul(GL_W, q[2]);
        }
    auto muls = [&](u32 lvl, u32 g) {
        PgMul m;
        for (u32 t = 0; t < PG_MAX_G * 10; t++) m.q[t] = t < g * 10 ? pr[10 * lvl + t] : 0;
        return m;
    };
    // the result comes back through a pinned block of the context's pool
    size_t res_bytes = 4096;
    while (res_bytes < std::max<size_t>(final_w, 1) * ew * 8) res_bytes <<= 1;
    u64* res = (u64*)effsc_internal_pinned_get(ctx, res_bytes);
    std::vector<u64> res_fallback;
    if (!res) {
        res_fallback.assign(res_bytes / 8, 0);
        res = res_fallback.data();
    }
    int rc = EFFSC_OK;
    u64 *d_in = nullptr, *bufs[2] = {nullptr, nullptr};
    const u64* cur = nullptr;
    if (width) {
        // device memory is read in place; host memory (pinned or pageable)
        // is copied first, so the passes only ever read device memory
        bool is_host = false;
        cur = effsc_internal_device_view(dev, polys, &is_host);
        if (is_host) cur = nullptr;
        if (!cur) {
            const size_t bytes = count0 * width * ew * 8;
            PCK(cudaMallocAsync((void**)&d_in, bytes, s));
            PCK(cudaMemcpyAsync(d_in, polys, bytes, cudaMemcpyHostToDevice, s));
            cur = d_in;
        }
    }
    if (K && width) {
        size_t count = count0;
        u32 w = (u32)width, lvl = 0;
        int which = 0;
        size_t cap[2] = {0, 0};
        static std::atomic<uint64_t> attr_done{0};    // one bit per device
        const uint64_t bit = 1ull << (dev & 63);
        if (!(attr_done.load() & bit)) {
            PCK(cudaFuncSetAttribute(k_pg_group<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PG_SMEM_BIG));
            PCK(cudaFuncSetAttribute(k_pg_group<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PG_SMEM_BIG));
            PCK(cudaFuncSetAttribute(k_pg_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(8 * PG_WARP_SMEM)));
            PCK(cudaFuncSetAttribute(k_pg_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(8 * PG_WARP_SMEM)));
            attr_done.fetch_or(bit);
        }
        while (count > 1) {
            const u32 gw = pg_plan_warp(count, w, ew);
            if (gw) {
                const size_t trees = count >> gw, need = trees * (w + gw) * ew * 8;
                if (need > cap[which]) {
                    if (bufs[which]) cudaFreeAsync(bufs[which], s);
                    bufs[which] = nullptr;
                    cap[which] = 0;
                    PCK(cudaMallocAsync((void**)&bufs[which], need, s));
                    cap[which] = need;
                }
                const size_t smem = (PG_TPB / 32) * pg_warp_smem(w, gw, ew);
                const unsigned grid = (unsigned)((trees + PG_TPB / 32 - 1) / (PG_TPB / 32));
                if (ew == 3) k_pg_warp<true><<<grid, PG_TPB, smem, s>>>(cur, trees, w, gw, muls(lvl, gw), bufs[which]);
                else k_pg_warp<false><<<grid, PG_TPB, smem, s>>>(cur, trees, w, gw, muls(lvl, gw), bufs[which]);
                effsc_internal_add_launches(1);
                PCK(cudaGetLastError());
                cur = bufs[which];
                which ^= 1;
                count = trees;
                w += gw;
                lvl += gw;
                continue;
            }
            u32 g = pg_plan_levels(count, w, ew, PG_SMEM);
            if (!g || (count >> g) < 4 * 152) g = std::max(g, pg_plan_levels(count, w, ew, PG_SMEM_BIG));
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
                const u32 S = pg_stride(w, g);
                if (ew == 3) k_pg_group<true><<<(unsigned)out_rows, PG_TPB, smem, s>>>(cur, w, g, S, muls(lvl, g), bufs[which]);
                else k_pg_group<false><<<(unsigned)out_rows, PG_TPB, smem, s>>>(cur, w, g, S, muls(lvl, g), bufs[which]);
                lvl += g;
            } else {
                const size_t items = out_rows * (w + 1);
                const unsigned grid = (unsigned)std::min<size_t>((items + PG_TPB - 1) / PG_TPB, 152 * 16);
                if (ew == 3) k_pg_level<true><<<grid, PG_TPB, 0, s>>>(cur, out_rows, w, muls(lvl, 1), bufs[which]);
                else k_pg_level<false><<<grid, PG_TPB, 0, s>>>(cur, out_rows, w, muls(lvl, 1), bufs[which]);
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
    if (final_w && width) PCK(cudaMemcpyAsync(res, cur, final_w * ew * 8, cudaMemcpyDefault, s));
    PCK(cudaStreamSynchronize(s));
    {
        size_t len = width ? final_w : 0;
        auto zero = [&](size_t e) {
            for (u32 c = 0; c < ew; c++)
                if (res[e * ew + c]) return false;
            return true;
        };
        const size_t keep = n_polys >= 2 ? 1 : 0;    // to_dense_poly keeps one term; a lone input is returned as is
        while (len > keep && zero(len - 1)) len--;
        if (n_polys >= 2 && len == 0) len = 1;       // width 0: the zero polynomial as one term
        for (size_t e = 0; e < len; e++)
            for (u32 c = 0; c < ew; c++) out[e * ew + c] = (width && e < final_w) ? res[e * ew + c] : 0;
        *out_len = len;
    }
done:
    for (void* p : {(void*)d_in, (void*)bufs[0], (void*)bufs[1]})
        if (p) cudaFreeAsync(p, s);
    if (res_fallback.empty()) effsc_internal_pinned_put(ctx, res, res_bytes);
    return rc;
}
