// k_misc.cu -- fold kernels, launch dispatch, and utility kernels (layout and
// representation conversion at the boundary, eq-table construction).
#include "round_common.cuh"

#include <atomic>
#include <cstdlib>

namespace effsc {

bool launch_eval_mlip(int pol, int sem, u32 mask, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_fused_mlip(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_eval_coef(int pol, int sem, u32 mask, const RoundArgs& a, int grid, cudaStream_t s);
bool launch_fused_coef(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s);

// SM count per device, read once per device (the attribute never changes, so
// concurrent first reads store the same value).  Grids are sized for the
// device current on the calling thread.
constexpr int SMS_MAX_DEVICES = 64;
static std::atomic<int> g_sms[SMS_MAX_DEVICES];

static int sms_of(int device) {
    if (device < 0 || device >= SMS_MAX_DEVICES) return 1;
    int v = g_sms[device].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0) v = 1;
        g_sms[device].store(v, std::memory_order_relaxed);
    }
    return v;
}

void kernels_init(int device) { sms_of(device); }

// Programmatic dependent launch of the round kernels: off unless EFFSC_PDL=1
// (measured at n = 26 in a CUDA graph: 1.273 ms per proof with it, 1.251
// without).
bool pdl_on(void) {
    static const bool on = [] {
        const char* e = getenv("EFFSC_PDL");
        return e && e[0] == '1';
    }();
    return on;
}
__global__ void k_gather_first(FirstSrc src, u64* dst) {
    chain_enter();
    const int i = threadIdx.x;
    if (i < 12) {
        const u64* p = src.p[i / 3][i % 3];
        dst[i] = p ? p[0] : 0;
    }
}
void launch_gather_first(const FirstSrc& src, u64* dst, cudaStream_t s) { launch_chain(k_gather_first, 1, 32, 0, s, src, dst); }

int max_grid(void) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    return sms_of(dev) * 8;
}

int pol_ntables(int pol) {
    switch (pol) {
    case POL_X1: case POL_X2: case POL_X3: return 4;
    case POL_ML: case POL_C1: return 1;
    case POL_C3: case POL_C3W: case POL_EQFL: return 3;
    case POL_GKR: return 4;
    default: return 2;
    }
}
int pol_nraw(int pol) {
    switch (pol) {
    case POL_X1: case POL_X2: case POL_X3: return 4;
    case POL_C2: case POL_C3W: return 3;
    case POL_C3: return 4;
    default: return 2;
    }
}
int pol_nwire(int pol) {
    switch (pol) {
    case POL_ML: case POL_C1: case POL_X1: return 1;
    case POL_X2: return 2;
    case POL_X3: return 3;
    case POL_C3: case POL_C3W: return 3;
    default: return 2;
    }
}

bool launch_eval(int pol, int sem, u32 mask, const RoundArgs& a, int grid, cudaStream_t s) {
    if (pol == POL_C1 || pol == POL_C2 || pol == POL_C3 || pol == POL_C3W) return launch_eval_coef(pol, sem, mask, a, grid, s);
    return launch_eval_mlip(pol, sem, mask, a, grid, s);
}
bool launch_fused(int pol, int sem, u32 mask, bool ech, const RoundArgs& a, int grid, cudaStream_t s) {
    if (pol == POL_C1 || pol == POL_C2 || pol == POL_C3 || pol == POL_C3W) return launch_fused_coef(pol, sem, mask, ech, a, grid, s);
    return launch_fused_mlip(pol, sem, mask, ech, a, grid, s);
}

#define FOLD(SEM, EI, ECH) \
    case ((SEM) * 4 + (EI) * 2 + (ECH)): return launch_chain(k_fold<SEM, EI, ECH>, grid, TPB, 0, s, a, t);

bool launch_fold(int sem, bool ein, bool ech, const RoundArgs& a, int t, int grid, cudaStream_t s) {
    if (ein) ech = true;
    switch (sem * 4 + (ein ? 2 : 0) + (ech ? 1 : 0)) {
        FOLD(SEM_MSB_PAD, false, false) FOLD(SEM_MSB_PAD, false, true) FOLD(SEM_MSB_PAD, true, true)
        FOLD(SEM_MSB_FLOOR, false, false) FOLD(SEM_MSB_FLOOR, false, true) FOLD(SEM_MSB_FLOOR, true, true)
        FOLD(SEM_LSB, false, false) FOLD(SEM_LSB, false, true) FOLD(SEM_LSB, true, true)
        default: return false;
    }
}

// ---------------------------------------------------------------------------
// Boundary conversion.  Montgomery residues of the crate (src/field.rs:314-375)
// are x * 2^64 mod p; canonical = mont * 2^-64 = mont * (p - 2^32) mod p.
// ---------------------------------------------------------------------------
#define R_INV (GL_P - (1ULL << 32))

__device__ __forceinline__ u64 canon_in(u64 x, int from_mont) {
    x = x >= GL_P ? x - GL_P : x;
    return from_mont ? gl_mul(x, R_INV) : x;
}

__global__ void k_split_aos(const u64* aos, u64 n, int ncomp, u64* c0, u64* c1, u64* c2,
                            int from_mont, u32* ext_flag) {
    u32 any = 0;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        if (ncomp == 1) {
            c0[i] = canon_in(aos[i], from_mont);
        } else {
            u64 x0 = canon_in(aos[3 * i], from_mont), x1 = canon_in(aos[3 * i + 1], from_mont),
                x2 = canon_in(aos[3 * i + 2], from_mont);
            c0[i] = x0;
            if (c1) { c1[i] = x1; c2[i] = x2; }
            any |= (x1 | x2) != 0;
        }
    }
    if (ext_flag && __any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) atomicOr(ext_flag, 1u);
}
void launch_split_aos(const u64* aos, u64 n, int ncomp, u64* c0, u64* c1, u64* c2, int from_mont,
                      u32* ext_flag, cudaStream_t s) {
    if (!n) return;
    u64 blocks = (n + 255) / 256;
    int g = (int)(blocks < (u64)max_grid() * 2 ? blocks : (u64)max_grid() * 2);
    k_split_aos<<<g, 256, 0, s>>>(aos, n, ncomp, c0, c1, c2, from_mont, ext_flag);
}

__global__ void k_join_aos(const u64* c0, const u64* c1, const u64* c2, u64 n, int ncomp, u64* aos, int to_mont) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        u64 x0 = c0[i], x1 = c1 ? c1[i] : 0, x2 = c2 ? c2[i] : 0;
        if (to_mont) { x0 = gl_mul(x0, GL_EPS); x1 = gl_mul(x1, GL_EPS); x2 = gl_mul(x2, GL_EPS); }
        if (ncomp == 1) aos[i] = x0;
        else { aos[3 * i] = x0; aos[3 * i + 1] = x1; aos[3 * i + 2] = x2; }
    }
}
void launch_join_aos(const u64* c0, const u64* c1, const u64* c2, u64 n, int ncomp, u64* aos, int to_mont,
                     cudaStream_t s) {
    if (!n) return;
    u64 blocks = (n + 255) / 256;
    int g = (int)(blocks < (u64)max_grid() * 2 ? blocks : (u64)max_grid() * 2);
    k_join_aos<<<g, 256, 0, s>>>(c0, c1, c2, n, ncomp, aos, to_mont);
}

__global__ void k_copy(const u64* src, u64* dst, u64 n) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) dst[i] = src[i];
}
void launch_copy(const u64* src, u64* dst, u64 n, cudaStream_t s) {
    if (!n) return;
    u64 blocks = (n + 255) / 256;
    int g = (int)(blocks < (u64)max_grid() * 2 ? blocks : (u64)max_grid() * 2);
    k_copy<<<g, 256, 0, s>>>(src, dst, n);
}
__global__ void k_fill(u64* dst, u64 n, u64 v) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) dst[i] = v;
}
void launch_fill(u64* dst, u64 n, u64 v, cudaStream_t s) {
    if (!n) return;
    u64 blocks = (n + 255) / 256;
    int g = (int)(blocks < (u64)max_grid() * 2 ? blocks : (u64)max_grid() * 2);
    k_fill<<<g, 256, 0, s>>>(dst, n, v);
}

// eq(w, x) over {0,1}^v in MSB layout (reference build_eq_table,
// src/provers/eq_factored.rs:217-239): entry idx = prod_j (bit_j ? w_j : 1 - w_j)
// with bit_j = bit (v-1-j) of idx.  Products are exact, so the order of the
// factors does not change the value.  w: v Fp3 values (AoS, canonical).
template <bool E>
__global__ void k_build_eq(const u64* w, u32 v, u64* c0, u64* c1, u64* c2) {
    const u64 n = 1ULL << v;
    for (u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (u64)gridDim.x * blockDim.x) {
        F3 acc = f3_make(1, 0, 0);
        for (u32 j = 0; j < v; j++) {
            F3 wj = f3_make(w[3 * j], w[3 * j + 1], w[3 * j + 2]);
            F3 f = ((idx >> (v - 1 - j)) & 1) ? wj : f3_sub<E>(f3_make(1, 0, 0), wj);
            acc = f3_mul<E, E>(acc, f);
        }
        c0[idx] = acc.c0;
        if (E) { c1[idx] = acc.c1; c2[idx] = acc.c2; }
    }
}
bool launch_build_eq(const u64* w, u32 v, int ext, u64* c0, u64* c1, u64* c2, cudaStream_t s) {
    u64 n = 1ULL << v;
    u64 blocks = (n + 255) / 256;
    int g = (int)(blocks < (u64)max_grid() * 2 ? blocks : (u64)max_grid() * 2);
    if (ext) k_build_eq<true><<<g, 256, 0, s>>>(w, v, c0, c1, c2);
    else k_build_eq<false><<<g, 256, 0, s>>>(w, v, c0, c1, c2);
    return true;
}

}  // namespace effsc

namespace effsc {

__device__ __forceinline__ u64 splitmix64_mix_dev(u64 z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
// Seeded uniform table: element i = SplitMix64 output i, re-mixed while >= p.
__global__ void k_gen_uniform(u64 seed, u64 n, u64* out) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        u64 z = splitmix64_mix_dev(seed + (i + 1) * 0x9E3779B97F4A7C15ULL);
        while (z >= GL_P) z = splitmix64_mix_dev(z + 0x9E3779B97F4A7C15ULL);
        out[i] = z;
    }
}
void launch_gen_uniform(u64 seed, u64 n, u64* out, cudaStream_t s) {
    if (!n) return;
    u64 blocks = (n + 255) / 256;
    int g = (int)(blocks < (u64)max_grid() * 2 ? blocks : (u64)max_grid() * 2);
    k_gen_uniform<<<g, 256, 0, s>>>(seed, n, out);
}

}  // namespace effsc

namespace effsc {

// Integer-pipe microbenchmark: CH independent chains per thread.
template <int CH>
__global__ void k_mulmod_chain(u64* out, u32 iters, u64 seed) {
    u64 x[CH];
    const u64 m = 0x9E3779B97F4A7C15ULL % GL_P;
    for (int c = 0; c < CH; c++) x[c] = (seed + threadIdx.x + 131 * blockIdx.x + 7 * c) % GL_P;
    for (u32 i = 0; i < iters; i++)
#pragma unroll
        for (int c = 0; c < CH; c++) x[c] = gl_mul(x[c], m);
    u64 r = 0;
    for (int c = 0; c < CH; c++) r ^= x[c];
    if (r == 0x1234567) out[0] = r;   // keeps the chains live
}
template <int CH>
__global__ void k_fp3_chain(u64* out, u32 iters, u64 seed) {
    F3 x[CH];
    const F3 m = f3_make(0x9E3779B97F4A7C15ULL % GL_P, 12345, 678910);
    const Mul3 mm = mul3_prepare<true>(m);
    for (int c = 0; c < CH; c++) x[c] = f3_make((seed + threadIdx.x + c) % GL_P, blockIdx.x, c);
    for (u32 i = 0; i < iters; i++)
#pragma unroll
        for (int c = 0; c < CH; c++) x[c] = f3_mul_add<true, true, false, false>(x[c], mm, f3_zero());
    u64 r = 0;
    for (int c = 0; c < CH; c++) r ^= x[c].c0 ^ x[c].c1 ^ x[c].c2;
    if (r == 0x1234567) out[0] = r;
}

// Accumulate-form rate: K independent lazy sums per thread, each new 64-bit
// operand multiplied by a per-sum constant and added unreduced -- the form of
// every fold and round-polynomial sum in the round kernels.  FORM 1 = the
// split accumulator of the folds, 0 = the 5-limb form of the long sums.
template <int FORM, int K>
__global__ void __launch_bounds__(256) k_accmac_chain(u64* out, u32 iters, u64 seed) {
    const u64 tid = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    u64 x = splitmix64_mix_dev(seed + tid);
    u64 y[K];
    AccF<FORM> a[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        y[k] = splitmix64_mix_dev(seed * 31 + k) % GL_P;
        a[k].zero();
    }
    for (u32 i = 0; i < iters; i++) {
        x += 0x9E3779B97F4A7C15ULL;
#pragma unroll
        for (int k = 0; k < K; k++) a[k].mac(x, y[k]);
    }
    u64 r = 0;
#pragma unroll
    for (int k = 0; k < K; k++) r ^= a[k].reduce();
    if (r == 0x1234567) out[0] = r;
}
// Reduction rate: one acc_reduce of a fresh 160-bit value per iteration.
__global__ void __launch_bounds__(256) k_reduce_chain(u64* out, u32 iters, u64 seed) {
    const u64 tid = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    u64 x = splitmix64_mix_dev(seed + tid), r = 0;
    for (u32 i = 0; i < iters; i++) {
        x += 0x9E3779B97F4A7C15ULL;
        Acc a;
        a.c0 = lo32(x); a.c1 = hi32(x); a.c2 = lo32(x) ^ i; a.c3 = hi32(x) + i; a.c4 = i & 7;
        r ^= acc_reduce(a);
    }
    if (r == 0x1234567) out[0] = r;
}

bool diag_accumulate_rate(cudaStream_t s, double* mac_per_s, double* reduce_per_s) {
    u64* out = nullptr;
    if (cudaMallocAsync((void**)&out, sizeof(u64), s) != cudaSuccess) return false;
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_accmac_chain<1, 2>, 256, 0) != cudaSuccess || bps < 1) bps = 1;
    const int blocks_mac = (max_grid() / 8) * bps;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_reduce_chain, 256, 0) != cudaSuccess || bps < 1) bps = 1;
    const int blocks_red = (max_grid() / 8) * bps;
    const u32 iters = 1u << 15;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float ms1 = 0, ms2 = 0;
    for (int rep = 0; rep < 2; rep++) {   // the first pass warms up
        cudaEventRecord(a, s);
        k_accmac_chain<1, 2><<<blocks_mac, 256, 0, s>>>(out, iters, 1);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms1, a, b);
        cudaEventRecord(a, s);
        k_reduce_chain<<<blocks_red, 256, 0, s>>>(out, iters, 1);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms2, a, b);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFreeAsync(out, s);
    bool ok = cudaStreamSynchronize(s) == cudaSuccess && ms1 > 0 && ms2 > 0;
    *mac_per_s = (double)blocks_mac * 256 * iters * 2 / (ms1 * 1e-3);
    *reduce_per_s = (double)blocks_red * 256 * iters / (ms2 * 1e-3);
    return ok;
}

bool diag_mulmod_rate(cudaStream_t s, double* mulmod_per_s, double* fp3_mul_per_s) {
    u64* out = nullptr;
    if (cudaMallocAsync((void**)&out, sizeof(u64), s) != cudaSuccess) return false;
    const int blocks = max_grid(), threads = 256;
    const u32 iters = 4096;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float ms1 = 0, ms2 = 0;
    for (int rep = 0; rep < 2; rep++) {   // the first pass warms up
        cudaEventRecord(a, s);
        k_mulmod_chain<8><<<blocks, threads, 0, s>>>(out, iters, 1);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms1, a, b);
        cudaEventRecord(a, s);
        k_fp3_chain<4><<<blocks, threads, 0, s>>>(out, iters / 4, 1);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms2, a, b);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFreeAsync(out, s);
    bool ok = cudaStreamSynchronize(s) == cudaSuccess && ms1 > 0 && ms2 > 0;
    double total_threads = (double)blocks * threads;
    *mulmod_per_s = total_threads * iters * 8 / (ms1 * 1e-3);
    *fp3_mul_per_s = total_threads * (iters / 4) * 4 / (ms2 * 1e-3);
    return ok;
}

}  // namespace effsc
