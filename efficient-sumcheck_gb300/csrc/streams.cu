// streams.cu -- the crate's evaluation streams on the device
// (src/streams/memory/core.rs, src/streams/stream.rs).
//
//   * reorder_vec_msb: out[i] = src[bit_reverse(i, num_vars)] -- ascending
//     (lexicographic) evaluations to the MSB (half-split) layout
//     (memory/core.rs:20-47); a gather kernel over device copies;
//   * multivariate_claim / multivariate_product_claim: sum over the hypercube
//     of one table / of the entrywise product of several (stream.rs:3-40);
//     the tables are read where they are, host memory included.
// Provers can also read their input tables in place from host memory
// (effsc_prover_create_host in runtime.cu): tables larger than HBM stay in
// host memory and only the folded tables live on the device.
#include "effsc_gpu.h"
#include "kernels.h"
#include "round_common.cuh"

#include <vector>

using namespace effsc;

int effsc_internal_ctx_device(const effsc_ctx* c);
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c);
uint64_t effsc_internal_add_launches(uint64_t k);
const u64* effsc_internal_device_view(int device, const uint64_t* ptr, bool* is_host);

namespace effsc {

__global__ void k_reorder_msb(const u64* src, u64* dst, u64 n, u32 v, int ncomp) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 j = v ? (__brevll(i) >> (64 - v)) : 0;
        for (int c = 0; c < ncomp; c++) dst[i * ncomp + c] = src[j * ncomp + c];
    }
}

struct ClaimTabs {
    const u64* t[4];
};

// partial[block] = sum over this block's entries of prod_t table_t[i]
template <bool E>
__global__ void __launch_bounds__(TPB) k_claim(ClaimTabs tabs, int nt, u64 n, int ncomp, u64* partial) {
    __shared__ u64 s_red[NWARP][3];
    SumAcc<E> acc;
    acc.init();
    for (u64 i = (u64)blockIdx.x * TPB + threadIdx.x; i < n; i += (u64)gridDim.x * TPB) {
        F3 p = ncomp == 3 ? f3_make(tabs.t[0][3 * i], tabs.t[0][3 * i + 1], tabs.t[0][3 * i + 2])
                          : f3_make(tabs.t[0][i], 0, 0);
        for (int t = 1; t < nt; t++) {
            const F3 x = ncomp == 3 ? f3_make(tabs.t[t][3 * i], tabs.t[t][3 * i + 1], tabs.t[t][3 * i + 2])
                                    : f3_make(tabs.t[t][i], 0, 0);
            p = f3_mul<E, E>(p, x);
        }
        acc.add(p);
    }
    F3 v = acc.result();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        v.c0 = gl_add(v.c0, __shfl_down_sync(0xffffffffu, v.c0, off));
        v.c1 = gl_add(v.c1, __shfl_down_sync(0xffffffffu, v.c1, off));
        v.c2 = gl_add(v.c2, __shfl_down_sync(0xffffffffu, v.c2, off));
    }
    if (lane == 0) { s_red[warp][0] = v.c0; s_red[warp][1] = v.c1; s_red[warp][2] = v.c2; }
    __syncthreads();
    if (threadIdx.x < 3) {
        u64 t = 0;
        for (int w = 0; w < NWARP; w++) t = gl_add(t, s_red[w][threadIdx.x]);
        partial[3 * blockIdx.x + threadIdx.x] = t;
    }
}

}  // namespace effsc

namespace {
const u64 HP = 0xFFFFFFFF00000001ULL;
u64 hadd(u64 a, u64 b) {
    u64 s = a + b;
    if (s < a || s >= HP) s -= HP;
    return s;
}
}  // namespace

#define SCK2(call)                                                                                          \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

extern "C" {

int effsc_reorder_msb(effsc_ctx* ctx, const uint64_t* src, size_t n, int ncomp, uint64_t* dst) {
    if (!ctx || !src || !dst) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    if (ncomp != 1 && ncomp != 3) return effsc_set_error(EFFSC_INVALID_ARG, "ncomp must be 1 or 3");
    // reorder_vec_msb asserts a non-empty power-of-two length (memory/core.rs:21)
    if (!n || (n & (n - 1))) return effsc_set_error(EFFSC_PANIC, "length %zu is not a power of two", n);
    const int dev = effsc_internal_ctx_device(ctx);
    cudaStream_t s = effsc_internal_ctx_stream(ctx);
    SCK2(cudaSetDevice(dev));
    u32 v = 0;
    while (((size_t)1 << v) < n) v++;
    const size_t bytes = n * (size_t)ncomp * sizeof(u64);
    u64* a = nullptr;
    u64* b = nullptr;
    SCK2(cudaMallocAsync((void**)&a, bytes, s));
    SCK2(cudaMallocAsync((void**)&b, bytes, s));
    SCK2(cudaMemcpyAsync(a, src, bytes, cudaMemcpyDefault, s));
    const u64 blocks = (n + 255) / 256;
    k_reorder_msb<<<(int)(blocks < (u64)max_grid() ? blocks : (u64)max_grid()), 256, 0, s>>>(a, b, n, v, ncomp);
    effsc_internal_add_launches(1);
    SCK2(cudaGetLastError());
    SCK2(cudaMemcpyAsync(dst, b, bytes, cudaMemcpyDefault, s));
    SCK2(cudaFreeAsync(a, s));
    SCK2(cudaFreeAsync(b, s));
    SCK2(cudaStreamSynchronize(s));
    return EFFSC_OK;
}

int effsc_stream_claim(effsc_ctx* ctx, int field, int n_tables, const uint64_t* const* tables, size_t n, int ncomp,
                       uint64_t* out) {
    if (!ctx || !tables || !out) return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    if (field != EFFSC_FP && field != EFFSC_FP3) return effsc_set_error(EFFSC_INVALID_ARG, "bad field");
    if (ncomp != 1 && ncomp != 3) return effsc_set_error(EFFSC_INVALID_ARG, "ncomp must be 1 or 3");
    // multivariate_product_claim asserts at least one stream (stream.rs:19)
    if (n_tables < 1 || n_tables > 4) return effsc_set_error(EFFSC_PANIC, "need 1 to 4 tables");
    const int dev = effsc_internal_ctx_device(ctx);
    cudaStream_t s = effsc_internal_ctx_stream(ctx);
    SCK2(cudaSetDevice(dev));
    ClaimTabs tabs = {{nullptr, nullptr, nullptr, nullptr}};
    for (int t = 0; t < n_tables; t++) {
        bool is_host = false;
        tabs.t[t] = tables[t] ? effsc_internal_device_view(dev, tables[t], &is_host) : nullptr;
        if (!tabs.t[t]) return effsc_set_error(EFFSC_UNSUPPORTED, "table %d: memory the GPU cannot read", t);
    }
    const u64 want = (n + TPB - 1) / TPB;
    const int g = (int)(want < 1 ? 1 : want < (u64)max_grid() ? want : (u64)max_grid());
    u64* part = nullptr;
    SCK2(cudaMallocAsync((void**)&part, (size_t)g * 3 * sizeof(u64), s));
    if (ncomp == 3 || field == EFFSC_FP3) k_claim<true><<<g, TPB, 0, s>>>(tabs, n_tables, n, ncomp, part);
    else k_claim<false><<<g, TPB, 0, s>>>(tabs, n_tables, n, ncomp, part);
    effsc_internal_add_launches(1);
    SCK2(cudaGetLastError());
    std::vector<u64> h((size_t)g * 3);
    SCK2(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(u64), cudaMemcpyDeviceToHost, s));
    SCK2(cudaFreeAsync(part, s));
    SCK2(cudaStreamSynchronize(s));
    u64 r[3] = {0, 0, 0};
    for (int b = 0; b < g; b++)
        for (int c = 0; c < 3; c++) r[c] = hadd(r[c], h[3 * b + c]);
    for (int c = 0; c < field; c++) out[c] = r[c];
    return EFFSC_OK;
}

}  // extern "C"
