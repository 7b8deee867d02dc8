// k_gkr_tail.cu -- the last rounds of a GkrProver proof in one thread block.
//
// Once add, mult, W_b and W_c fit in shared memory together, a round's kernel
// boundaries (the fold of W_b or W_c, the round kernel, the grid ticket and a
// lone last block running the transcript) cost more than its arithmetic.
// This kernel loads the four tables once (base tables embedded when the field
// is Fp3) and runs each round as the per-round path does
// (src/provers/gkr.rs:105-190): fold the witness table of the variable just
// bound and the gate tables with the previous challenge (MSB, in place),
// accumulate q(0) and the x^2 coefficient c2 over the pairs (i, i + H) as
// k_gkr.cu does, reduce across the block and run the transcript step in warp
// 0.  Then the runner's finalize (src/provers/gkr.rs:193-198: the gate tables
// and the witness table of the last variable folded once more), the tables'
// first entries for the read-back, and the tables written back so that the
// post-state accessors see what the per-round path leaves.
#include "round_common.cuh"

namespace effsc {

constexpr int GT_TPB = 256;   // 162 registers, no spills (512 threads: 128 and a spill; measured 0.795 vs 0.786 ms per k = 12 proof)
constexpr int GT_NW = GT_TPB / 32;

// Table t, component c, entry i at tb[t][c * st[t] + i]; st = starting length.
template <int FW>
struct GtTables {
    u64* tb[4];
    u64 st[4];
    __device__ __forceinline__ F3 ld(int t, u64 i) const {
        F3 r;
        r.c0 = tb[t][i];
        if (FW == 3) { r.c1 = tb[t][st[t] + i]; r.c2 = tb[t][2 * st[t] + i]; }
        else { r.c1 = r.c2 = 0; }
        return r;
    }
    __device__ __forceinline__ void put(int t, u64 i, const F3& v) const {
        tb[t][i] = v.c0;
        if (FW == 3) { tb[t][st[t] + i] = v.c1; tb[t][2 * st[t] + i] = v.c2; }
    }
    // new[j] = lo + (hi - lo) r over pairs (j, j + len/2); thread j alone
    // reads and writes entry j, so the fold runs in place.
    __device__ __forceinline__ void fold(int t, u64& len, const Mul3& m) const {
        if (len < 2) return;
        const u64 half = len >> 1;
        for (u64 j = threadIdx.x; j < half; j += GT_TPB) put(t, j, f3_fold<FW == 3, FW == 3>(ld(t, j), ld(t, j + half), m));
        len = half;
    }
};

template <int FW>
__global__ void __launch_bounds__(GT_TPB, 1) k_gkr_tail(GkrTailArgs a) {
    constexpr bool E = FW == 3;
    extern __shared__ __align__(16) u64 sm[];
    __shared__ u64 s_red[GT_NW][6];
    __shared__ u64 s_tot[6];
    __shared__ u64 s_chal[3];
    __shared__ __align__(8) uint8_t s_scr[64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    GtTables<FW> T;
    u64 len[4];
    u64 off = 0;
    for (int t = 0; t < 4; t++) {
        T.tb[t] = sm + off;
        T.st[t] = len[t] = a.len[t];
        off += (u64)FW * a.len[t];
    }
    for (int t = 0; t < 4; t++)
        for (int c = 0; c < FW; c++) {
            const u64* src = (c == 0 || ((a.in_ext >> t) & 1u)) ? a.in[t][c] : nullptr;
            u64* dst = T.tb[t] + (u64)c * T.st[t];
            for (u64 i = threadIdx.x; i < len[t]; i += GT_TPB) dst[i] = src ? src[i] : 0;
        }
    if (threadIdx.x < 3) s_chal[threadIdx.x] = a.first_fold ? a.chal_in[threadIdx.x] : 0;
    WarpTx w;
    if (warp == 0) w = tx_load((const DevTranscript*)a.tx, lane);
    __syncthreads();
    for (u32 j = 0; j < a.nrounds; j++) {
        if (j > 0 || a.first_fold) {
            const Mul3 m = mul3_prepare<E>(f3_make(s_chal[0], s_chal[1], s_chal[2]));
            const u32 prev = a.r0 + j - 1;                 // the variable just bound
            T.fold(0, len[0], m);
            T.fold(1, len[1], m);
            T.fold(prev < a.k ? 2 : 3, len[prev < a.k ? 2 : 3], m);
            __syncthreads();
        }
        ProdAcc<E, E> q0, qc;
        q0.init();
        qc.init();
        const u64 Ln = len[0];
        if (Ln == 1) {
            // q(1) = 0 and q(2) = -q(0): the wire's q(inf) is 0 (src/provers/gkr.rs:119-127)
            if (threadIdx.x == 0) {
                const F3 wb = T.ld(2, 0), wc = T.ld(3, 0);
                q0.mac(T.ld(0, 0), f3_add<E>(wb, wc));
                q0.mac(T.ld(1, 0), f3_mul<E, E>(wb, wc));
            }
        } else {
            const u32 lg = 63 - __clzll(Ln);
            const u32 kc = a.k < lg ? a.k : lg;
            const u64 cm = (1ULL << kc) - 1, H = Ln >> 1;
            const bool bvar = kc < lg;
            for (u64 i = threadIdx.x; i < H; i += GT_TPB) {
                const F3 al = T.ld(0, i), ah = T.ld(0, i + H), ml = T.ld(1, i), mh = T.ld(1, i + H);
                const F3 wbl = T.ld(2, i >> kc), wcl = T.ld(3, i & cm);
                q0.mac(al, f3_add<E>(wbl, wcl));
                q0.mac(ml, f3_mul<E, E>(wbl, wcl));
                const F3 da = f3_sub<E>(ah, al), dm = f3_sub<E>(mh, ml);
                if (bvar) qc.mac(f3_add<E>(f3_mul<E, E>(dm, wcl), da), f3_sub<E>(T.ld(2, (i + H) >> kc), wbl));
                else qc.mac(f3_add<E>(f3_mul<E, E>(dm, wbl), da), f3_sub<E>(T.ld(3, (i + H) & cm), wcl));
            }
        }
        F3 raw[2] = {q0.result(), qc.result()};
#pragma unroll
        for (int o = 16; o; o >>= 1)
#pragma unroll
            for (int v = 0; v < 2; v++) {
                raw[v].c0 = gl_add(raw[v].c0, __shfl_down_sync(0xffffffffu, raw[v].c0, o));
                raw[v].c1 = gl_add(raw[v].c1, __shfl_down_sync(0xffffffffu, raw[v].c1, o));
                raw[v].c2 = gl_add(raw[v].c2, __shfl_down_sync(0xffffffffu, raw[v].c2, o));
            }
        if (lane == 0) {
            s_red[warp][0] = raw[0].c0; s_red[warp][1] = raw[0].c1; s_red[warp][2] = raw[0].c2;
            s_red[warp][3] = raw[1].c0; s_red[warp][4] = raw[1].c1; s_red[warp][5] = raw[1].c2;
        }
        __syncthreads();
        if (warp == 0) {
            if (lane < 6) {
                u64 v = 0;
                for (int q = 0; q < GT_NW; q++) v = gl_add(v, s_red[q][lane]);
                s_tot[lane] = v;
            }
            __syncwarp();
            // transcript step (src/runner.rs:39-55): wire [q(0), q(inf)], hook, challenge
            tx_send_elems(w, lane, s_tot, 2);
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
            if (lane < 6) a.proof_wire[(u64)j * 6 + lane] = s_tot[lane];
            if (lane < 3) a.proof_chal[(u64)j * 3 + lane] = s_chal[lane];
        }
        __syncthreads();
    }
    if (warp == 0) tx_store((DevTranscript*)a.tx, w, lane);
    if (a.final_fold) {
        const Mul3 m = mul3_prepare<E>(f3_make(s_chal[0], s_chal[1], s_chal[2]));
        const u32 last = a.r0 + a.nrounds - 1;
        T.fold(0, len[0], m);
        T.fold(1, len[1], m);
        T.fold(last < a.k ? 2 : 3, len[last < a.k ? 2 : 3], m);
        __syncthreads();
    }
    if (a.first_out && threadIdx.x < 12) {
        const int t = threadIdx.x / 3, c = threadIdx.x % 3;
        a.first_out[threadIdx.x] = c < FW ? T.tb[t][(u64)c * T.st[t]] : 0;
    }
    for (int t = 0; t < 4; t++)
        if (a.out[t][0])
            for (int c = 0; c < FW; c++) {
                const u64* src = T.tb[t] + (u64)c * T.st[t];
                for (u64 i = threadIdx.x; i < len[t]; i += GT_TPB) a.out[t][c][i] = src[i];
            }
}

bool launch_gkr_tail(int fw, const GkrTailArgs& a, u64 smem_bytes, cudaStream_t s) {
    if (smem_bytes > TAIL_SMEM_CAP) return false;
    if (fw == 3) {
        cudaFuncSetAttribute(k_gkr_tail<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        k_gkr_tail<3><<<1, GT_TPB, smem_bytes, s>>>(a);
    } else {
        cudaFuncSetAttribute(k_gkr_tail<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_CAP);
        k_gkr_tail<1><<<1, GT_TPB, smem_bytes, s>>>(a);
    }
    return true;
}

}  // namespace effsc
