// k_persist.cu -- consecutive InnerProduct rounds over Fp3 tables in one
// cooperative launch.
//
// Once the tables are a few hundred MB or less, a round's pass takes a few
// microseconds and the per-launch costs (the launch itself, the ramp of a
// fresh grid, the grid ticket, a lone last block running the transcript step
// while the rest of the GPU idles) dominate: each such round cost 16-27 us.
// Here one grid of co-resident blocks runs the rounds back to back: per
// round, every block folds its share of the quadruples with the previous
// challenge (MSB (q, q+2Q), (q+Q, q+3Q) in place; LSB (4q, 4q+1),
// (4q+2, 4q+3) into the other of two buffers) and accumulates the next round
// polynomial (the same per-pair policy as the single-round kernels,
// src/provers/inner_product.rs:61-113), writes its partial sums and arrives
// at a grid barrier.  Block 0 waits for the others, sums the partials,
// builds the wire, runs the transcript step (absorb, hook, squeeze;
// src/runner.rs:39-55) and only then releases the barrier, so the next round
// starts with its challenge in memory.  Data written by other blocks of the same launch is
// read through L2 (ld.cg) and written through to it (st.cg).
// The barrier's waits are bounded (1 s of the global timer): a block that
// gives up records EFFSC_STATUS_TIMEOUT and returns, and so do the others
// at their next wait.  Every block is resident at once (a cooperative
// launch), so block 0's wait for the others ends.
#include "round_common.cuh"

namespace effsc {

__device__ __forceinline__ u32 ld_volatile_u32(const u32* p) { return *(const volatile u32*)p; }

// Round k of the launch; PAR = which ping-pong buffer it reads (LSB: k & 1,
// MSB: 0), a compile-time index so that the table pointers come straight
// from the kernel's parameters.  Returns false after a barrier timeout.
template <bool LSB, int PAR>
__device__ __forceinline__ bool persist_round(const RoundArgs& a, const PersistArgs& p, u32 k) {
    using P = Policy<POL_IP, 3>;
    constexpr int SRC = LSB ? PAR : 0, DST = LSB ? 1 - PAR : 0;
    __shared__ int s_flag;
    __shared__ u64 s_red[NWARP][6];
    __shared__ u64 s_tot[RAW_WORDS];
    const u32 nb = gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 tid = (u64)blockIdx.x * TPB + threadIdx.x, stride = (u64)nb * TPB;
    const u64 L = p.L0 >> k, Q = L >> 2;
    const u64* chp = k == 0 ? p.chal_in : p.proof_chal + 3 * (k - 1);
    const F3 r = f3_make(__ldcg(chp), __ldcg(chp + 1), __ldcg(chp + 2));
    const Mul3 rm = mul3_prepare<true>(r);
    P acc;
    acc.init();
    F3 lo[2], hi[2];
    for (u64 q = tid; q < Q; q += stride) {
#pragma unroll
        for (int t = 0; t < 2; t++) {
            const u64* const* in = p.buf[SRC][t];
            u64* const* out = p.buf[DST][t];
            if (LSB) {
                // two 16-byte loads per component
                ulonglong2 v[3][2];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    v[c][0] = __ldcg(reinterpret_cast<const ulonglong2*>(in[c] + 4 * q));
                    v[c][1] = __ldcg(reinterpret_cast<const ulonglong2*>(in[c] + 4 * q + 2));
                }
                lo[t] = f3_fold<true, true>(f3_make(v[0][0].x, v[1][0].x, v[2][0].x),
                                            f3_make(v[0][0].y, v[1][0].y, v[2][0].y), rm);
                hi[t] = f3_fold<true, true>(f3_make(v[0][1].x, v[1][1].x, v[2][1].x),
                                            f3_make(v[0][1].y, v[1][1].y, v[2][1].y), rm);
                __stcg(reinterpret_cast<ulonglong2*>(out[0] + 2 * q), make_ulonglong2(lo[t].c0, hi[t].c0));
                __stcg(reinterpret_cast<ulonglong2*>(out[1] + 2 * q), make_ulonglong2(lo[t].c1, hi[t].c1));
                __stcg(reinterpret_cast<ulonglong2*>(out[2] + 2 * q), make_ulonglong2(lo[t].c2, hi[t].c2));
            } else {
                F3 x[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const u64 e = q + j * Q;
                    x[j] = f3_make(__ldcg(in[0] + e), __ldcg(in[1] + e), __ldcg(in[2] + e));
                }
                lo[t] = f3_fold<true, true>(x[0], x[2], rm);
                hi[t] = f3_fold<true, true>(x[1], x[3], rm);
                __stcg(out[0] + q, lo[t].c0);
                __stcg(out[1] + q, lo[t].c1);
                __stcg(out[2] + q, lo[t].c2);
                __stcg(out[0] + q + Q, hi[t].c0);
                __stcg(out[1] + q + Q, hi[t].c1);
                __stcg(out[2] + q + Q, hi[t].c2);
            }
        }
        acc.pair(lo, hi);
    }
    // the block's partial sums
    F3 raw[P::NRAW];
    acc.result(raw);
#pragma unroll
    for (int off = 16; off; off >>= 1)
#pragma unroll
        for (int i = 0; i < 2; i++) {
            raw[i].c0 = gl_add(raw[i].c0, __shfl_down_sync(0xffffffffu, raw[i].c0, off));
            raw[i].c1 = gl_add(raw[i].c1, __shfl_down_sync(0xffffffffu, raw[i].c1, off));
            raw[i].c2 = gl_add(raw[i].c2, __shfl_down_sync(0xffffffffu, raw[i].c2, off));
        }
    if (lane == 0)
        for (int i = 0; i < 2; i++) {
            s_red[warp][3 * i] = raw[i].c0;
            s_red[warp][3 * i + 1] = raw[i].c1;
            s_red[warp][3 * i + 2] = raw[i].c2;
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        u64 v = 0;
#pragma unroll
        for (int w = 0; w < NWARP; w++) v = gl_add(v, s_red[w][threadIdx.x]);
        a.partials[(u64)blockIdx.x * RAW_WORDS + threadIdx.x] = v;
    }
    // arrive: block 0 waits for the others, finalises the round and releases
    // them (always the same block, so that the transcript code stays in one
    // SM's instruction cache across the rounds)
    __threadfence();
    __syncthreads();
    bool ok = true;
    if (blockIdx.x != 0) {
        if (threadIdx.x == 0) {
            const u32 g0 = ld_volatile_u32(p.bar + 1);
            __threadfence();
            atomicAdd(p.bar, 1u);
            bool done = true;
            if (ld_volatile_u32(p.bar + 1) == g0) {
                const u64 t0 = global_ns();
                while (ld_volatile_u32(p.bar + 1) == g0)
                    if (global_ns() - t0 > 1000000000ULL) { done = false; break; }
            }
            s_flag = done ? 0 : -1;
            if (!done && a.status) *(volatile u32*)a.status = EFFSC_STATUS_TIMEOUT;
            __threadfence();
        }
        __syncthreads();
        ok = s_flag >= 0;
    } else {
        if (threadIdx.x == 0) {
            bool done = true;
            if (ld_volatile_u32(p.bar) != nb - 1) {
                const u64 t0 = global_ns();
                while (ld_volatile_u32(p.bar) != nb - 1)
                    if (global_ns() - t0 > 1000000000ULL) { done = false; break; }
            }
            s_flag = done ? 0 : -1;
            if (!done && a.status) *(volatile u32*)a.status = EFFSC_STATUS_TIMEOUT;
            __threadfence();
        }
        __syncthreads();
        if (s_flag < 0) return false;
        // every thread walks a stride of the blocks' partials, then warp and
        // block sums
        u64 t6[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 2
        for (u32 b = threadIdx.x; b < nb; b += TPB)
#pragma unroll
            for (int i = 0; i < 6; i++) t6[i] = gl_add(t6[i], __ldcg(&a.partials[(u64)b * RAW_WORDS + i]));
#pragma unroll
        for (int off = 16; off; off >>= 1)
#pragma unroll
            for (int i = 0; i < 6; i++) t6[i] = gl_add(t6[i], __shfl_down_sync(0xffffffffu, t6[i], off));
        __syncthreads();
        if (lane == 0)
#pragma unroll
            for (int i = 0; i < 6; i++) s_red[warp][i] = t6[i];
        __syncthreads();
        if (threadIdx.x < 6) {
            u64 v = 0;
#pragma unroll
            for (int w = 0; w < NWARP; w++) v = gl_add(v, s_red[w][threadIdx.x]);
            s_tot[threadIdx.x] = v;
        } else if (threadIdx.x < RAW_WORDS) {
            s_tot[threadIdx.x] = 0;
        }
        __syncthreads();
        if (warp == 0) {
            RoundArgs fa = a;
            fa.tx.proof_wire = p.proof_wire + 6 * k;
            fa.tx.proof_chal = p.proof_chal + 3 * k;
            fa.tx.chal_next = nullptr;
            finalize_warp(POL_IP, s_tot, fa);
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            *(volatile u32*)p.bar = 0;
            __threadfence();
            atomicAdd(p.bar + 1, 1u);
        }
    }
    __syncthreads();
    return ok;
}

template <bool LSB>
__global__ void __launch_bounds__(TPB, 2) k_ip_persist(RoundArgs a, PersistArgs p) {
    chain_enter();
    for (u32 k = 0; k < p.nrounds; k += 2) {
        if (!persist_round<LSB, 0>(a, p, k)) return;
        if (k + 1 < p.nrounds && !persist_round<LSB, 1>(a, p, k + 1)) return;
    }
}

// Co-resident blocks for the launch (a cooperative launch needs every block
// resident at once).
int persist_max_grid(bool lsb) {
    int bps = 0;
    cudaError_t e = lsb ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_ip_persist<true>, TPB, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_ip_persist<false>, TPB, 0);
    if (e != cudaSuccess || bps < 1) { cudaGetLastError(); return 0; }
    return bps * (max_grid() / 8);
}

bool launch_ip_persist(bool lsb, const RoundArgs& a, const PersistArgs& p, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(TPB, 1, 1);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return (lsb ? cudaLaunchKernelEx(&cfg, k_ip_persist<true>, a, p)
                : cudaLaunchKernelEx(&cfg, k_ip_persist<false>, a, p)) == cudaSuccess;
}

}  // namespace effsc
