// k_eqf.cu -- EqFactoredProver's left phase from the inner sums.
//
// In the left phase (src/provers/eq_factored.rs:139-172) every round's sums
// are inner products of the folded eq_l with the inner sums
//   S[a] = sum_b eq_r[b] p[a m + b]          (m = |eq_r|),
// and folding p over its left variables folds S the same way (the fold is
// linear and eq_r does not change), so the v_l left rounds are exactly
// InnerProduct rounds on the pair (eq_l, S) of 2^v_l entries: one pass over p
// for S (k_eqf_inner), then the one-block tail kernel for all left rounds.
// The folded p the right phase needs is p folded by the left challenges
// r_0 .. r_{v_l-2}: a weighted sum of its 2^(v_l-1) row blocks with the eq
// weights of those challenges (k_eqf_fold_rows + k_eqf_fold_sum), a second
// read of p instead of v_l - 1 read-and-write passes.
#include "round_common.cuh"

namespace effsc {

// S[a] for a = blockIdx.x (grid-stride): one block reduces one row of p.
template <bool EE, bool EP>
__global__ void __launch_bounds__(TPB) k_eqf_inner(Tab3 p, Tab3 er, u64 m, u64 rows, u64* s0, u64* s1, u64* s2) {
    __shared__ u64 s_red[NWARP][3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (u64 a = blockIdx.x; a < rows; a += gridDim.x) {
        ProdAcc<EE, EP> acc;
        acc.init();
#pragma unroll 8
        for (u64 b = threadIdx.x; b < m; b += TPB) acc.mac(ld<EE>(er.c, b), ld<EP>(p.c, a * m + b));
        F3 v = acc.result();
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
            u64* dst = threadIdx.x == 0 ? s0 : threadIdx.x == 1 ? s1 : s2;
            if (dst) dst[a] = t;
        }
        __syncthreads();
    }
}

// partial[split][c] = sum over rows a of split `split` of e[a] * p[a Lc + c]
// (block (tile, split): columns tile*TPB .. +TPB, rows split*per .. +per).
template <bool EW, bool EP>
__global__ void __launch_bounds__(TPB) k_eqf_fold_rows(Tab3 p, Tab3 e, u64 Lc, u64 rows, u64 per, u64 tiles, u64* part) {
    const u64 tile = blockIdx.x % tiles, split = blockIdx.x / tiles;
    const u64 c = tile * TPB + threadIdx.x;
    if (c >= Lc) return;
    ProdAcc<EW, EP> acc;
    acc.init();
    const u64 a0 = split * per, a1 = a0 + per < rows ? a0 + per : rows;
#pragma unroll 8
    for (u64 a = a0; a < a1; a++) acc.mac(ld<EW>(e.c, a), ld<EP>(p.c, a * Lc + c));
    const F3 v = acc.result();
    u64* dst = part + 3 * (split * Lc + c);
    dst[0] = v.c0;
    dst[1] = v.c1;
    dst[2] = v.c2;
}

// out[c] = sum over splits of partial[split][c] (FW components written).
__global__ void k_eqf_fold_sum(const u64* part, u64 Lc, u64 splits, int fw, u64* o0, u64* o1, u64* o2) {
    for (u64 c = (u64)blockIdx.x * blockDim.x + threadIdx.x; c < Lc; c += (u64)gridDim.x * blockDim.x) {
        u64 v0 = 0, v1 = 0, v2 = 0;
        for (u64 sp = 0; sp < splits; sp++) {
            const u64* src = part + 3 * (sp * Lc + c);
            v0 = gl_add(v0, src[0]);
            v1 = gl_add(v1, src[1]);
            v2 = gl_add(v2, src[2]);
        }
        o0[c] = v0;
        if (fw == 3) { o1[c] = v1; o2[c] = v2; }
    }
}

void launch_eqf_inner(bool ee, bool ep, Tab3 p, Tab3 er, u64 m, u64 rows, u64* s0, u64* s1, u64* s2, cudaStream_t s) {
    const int g = (int)(rows < (u64)max_grid() ? rows : (u64)max_grid());
    if (ee && ep) k_eqf_inner<true, true><<<g, TPB, 0, s>>>(p, er, m, rows, s0, s1, s2);
    else if (ee) k_eqf_inner<true, false><<<g, TPB, 0, s>>>(p, er, m, rows, s0, s1, s2);
    else if (ep) k_eqf_inner<false, true><<<g, TPB, 0, s>>>(p, er, m, rows, s0, s1, s2);
    else k_eqf_inner<false, false><<<g, TPB, 0, s>>>(p, er, m, rows, s0, s1, s2);
}

void launch_eqf_fold_rows(bool ew, bool ep, Tab3 p, Tab3 e, u64 Lc, u64 rows, u64 splits, u64* part, int fw, u64* o0,
                          u64* o1, u64* o2, cudaStream_t s) {
    const u64 tiles = (Lc + TPB - 1) / TPB, per = (rows + splits - 1) / splits;
    const int g = (int)(tiles * splits);
    if (ew && ep) k_eqf_fold_rows<true, true><<<g, TPB, 0, s>>>(p, e, Lc, rows, per, tiles, part);
    else if (ew) k_eqf_fold_rows<true, false><<<g, TPB, 0, s>>>(p, e, Lc, rows, per, tiles, part);
    else if (ep) k_eqf_fold_rows<false, true><<<g, TPB, 0, s>>>(p, e, Lc, rows, per, tiles, part);
    else k_eqf_fold_rows<false, false><<<g, TPB, 0, s>>>(p, e, Lc, rows, per, tiles, part);
    const u64 blocks = (Lc + TPB - 1) / TPB;
    k_eqf_fold_sum<<<(int)(blocks < (u64)max_grid() ? blocks : (u64)max_grid()), TPB, 0, s>>>(part, Lc, splits, fw, o0, o1, o2);
}

}  // namespace effsc
