// verify.cu -- sumcheck_verify (src/verifier.rs:61-139) for many proofs at
// once: one warp per proof replays the proof's transcript (receive the wire
// values, absorb the hook bytes, squeeze the challenge) and updates the claim
// from the EvalsInfty values:
//   h(1) = claim - h(0); h(inf) = recv[1] (degree >= 2) or h(1) - h(0);
//   q = [h(0), h(1) - h(inf), h(2) - 8 h(inf)] over {0, .., d-1};
//   claim = q(r) + h(inf) r^d,  q(r) by Lagrange interpolation.
// The final claims come back for the caller's oracle check (final_claim ==
// g(r)); for proofs made here that is the proof's final value.
#include "effsc_gpu.h"
#include "kernels.h"
#include "round_common.cuh"

#include <vector>

using namespace effsc;

int effsc_internal_ctx_device(const effsc_ctx* c);
cudaStream_t effsc_internal_ctx_stream(const effsc_ctx* c);
uint64_t effsc_internal_add_launches(uint64_t k);
void effsc_internal_tx_state(const effsc_transcript* t, void* out);

namespace effsc {

struct VerifyArgs {
    const u64* claimed;       // 3 words per proof
    const u64* polys;         // 3 words per element, degree elements per row
    const u64* row_off;       // first row of proof i
    const u32* rounds;        // rounds of proof i
    DevTranscript* tx;        // one per proof (state at the start)
    const uint8_t* hook;
    u32 hook_len;
    u32 degree;
    u32 n;
    u64* challenges;          // 3 words per row (optional)
    u64* finals;              // 3 words per proof
};

__global__ void k_verify_batch(VerifyArgs a) {
    __shared__ u64 s_wire[4][9];
    __shared__ u64 s_chal[4][3];
    __shared__ __align__(8) uint8_t s_scr[4][64];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const u32 i = blockIdx.x * 4 + wib;
    if (i >= a.n) return;
    const u32 d = a.degree, nw = d > 1 ? d : 1;
    WarpTx w = tx_load(a.tx + i, lane);
    F3 claim = f3_make(a.claimed[3 * i], a.claimed[3 * i + 1], a.claimed[3 * i + 2]);
    const u64 row0 = a.row_off[i];
    for (u32 rd = 0; rd < a.rounds[i]; rd++) {
        const u64* src = a.polys + (row0 + rd) * 3 * nw;
        if (lane < 3 * (int)nw) s_wire[wib][lane] = src[lane];
        __syncwarp();
        tx_send_elems(w, lane, s_wire[wib], (int)nw);
        if (a.hook_len) {
            const uint8_t* hk = a.hook;
            tx_absorb(w, lane, a.hook_len, [&](u32 k) -> uint8_t { return hk[k]; });
        }
        tx_challenge(w, lane, s_chal[wib], s_scr[wib]);
        if (lane == 0) {
            const F3 r = f3_make(s_chal[wib][0], s_chal[wib][1], s_chal[wib][2]);
            const F3 h0 = f3_make(s_wire[wib][0], s_wire[wib][1], s_wire[wib][2]);
            const F3 h1 = f3_sub<true>(claim, h0);
            if (d == 0) {
                claim = h0;
            } else {
                const F3 hinf = d >= 2 ? f3_make(s_wire[wib][3], s_wire[wib][4], s_wire[wib][5]) : f3_sub<true>(h1, h0);
                const F3 q0 = h0, q1 = f3_sub<true>(h1, hinf);
                F3 qr, rd_pow = r;
                if (d <= 2) {
                    qr = f3_add<true>(q0, f3_mul<true, true>(r, f3_sub<true>(q1, q0)));
                    if (d == 2) rd_pow = f3_mul<true, true>(r, r);
                } else {
                    // q2 = h(2) - 8 h(inf); Lagrange over {0, 1, 2}:
                    // q(r) = q0 (r-1)(r-2)/2 - q1 r (r-2) + q2 r (r-1)/2
                    const F3 h2 = f3_make(s_wire[wib][6], s_wire[wib][7], s_wire[wib][8]);
                    F3 h8 = f3_add<true>(hinf, hinf);
                    h8 = f3_add<true>(h8, h8);
                    h8 = f3_add<true>(h8, h8);
                    const F3 q2 = f3_sub<true>(h2, h8);
                    const F3 one = f3_make(1, 0, 0), two = f3_make(2, 0, 0);
                    const F3 rm1 = f3_sub<true>(r, one), rm2 = f3_sub<true>(r, two);
                    const u64 inv2 = 0x7FFFFFFF80000001ULL;
                    F3 t0 = f3_mul<true, true>(f3_mul<true, true>(rm1, rm2), q0);
                    F3 t2 = f3_mul<true, true>(f3_mul<true, true>(r, rm1), q2);
                    F3 half = f3_add<true>(t0, t2);
                    half = f3_make(gl_mul(half.c0, inv2), gl_mul(half.c1, inv2), gl_mul(half.c2, inv2));
                    qr = f3_sub<true>(half, f3_mul<true, true>(f3_mul<true, true>(r, rm2), q1));
                    rd_pow = f3_mul<true, true>(f3_mul<true, true>(r, r), r);
                }
                claim = f3_add<true>(qr, f3_mul<true, true>(hinf, rd_pow));
            }
            if (a.challenges) {
                u64* c = a.challenges + (row0 + rd) * 3;
                c[0] = r.c0; c[1] = r.c1; c[2] = r.c2;
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        a.finals[3 * i] = claim.c0;
        a.finals[3 * i + 1] = claim.c1;
        a.finals[3 * i + 2] = claim.c2;
    }
}

}  // namespace effsc

#define VCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) { rc = effsc_set_error(EFFSC_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); goto done; } \
    } while (0)

extern "C" int effsc_verify_batch(effsc_ctx* ctx, int field, size_t n, const uint64_t* claimed_sums, int degree,
                                  const uint32_t* num_rounds, const effsc_transcript* const* transcripts,
                                  const uint8_t* hook, size_t hook_len, const uint64_t* round_polys,
                                  uint64_t* challenges, uint64_t* final_claims) {
    if (!ctx || !claimed_sums || !num_rounds || !transcripts || !final_claims || (hook_len && !hook))
        return effsc_set_error(EFFSC_INVALID_ARG, "NULL argument");
    if (field != EFFSC_FP && field != EFFSC_FP3) return effsc_set_error(EFFSC_INVALID_ARG, "bad field");
    if (degree < 0 || degree > 3) return effsc_set_error(EFFSC_UNSUPPORTED, "device verification handles degree 0..3");
    if (hook_len >= (1ull << 32) || n >= (1ull << 32)) return effsc_set_error(EFFSC_INVALID_ARG, "hook or batch too large");
    if (!n) return EFFSC_OK;
    const int dev = effsc_internal_ctx_device(ctx);
    cudaStream_t s = effsc_internal_ctx_stream(ctx);
    if (cudaSetDevice(dev) != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "cudaSetDevice");
    const u32 nw = degree > 1 ? degree : 1;
    std::vector<u64> row_off(n + 1, 0), claimed(3 * n, 0);
    std::vector<DevTranscript> tx(n);
    for (size_t i = 0; i < n; i++) {
        row_off[i + 1] = row_off[i] + num_rounds[i];
        for (int c = 0; c < field; c++) claimed[3 * i + c] = claimed_sums[i * field + c] % 0xFFFFFFFF00000001ULL;
        if (!transcripts[i]) return effsc_set_error(EFFSC_INVALID_ARG, "transcript %zu is NULL", i);
        effsc_internal_tx_state(transcripts[i], &tx[i]);
        if ((int)tx[i].deg != field) return effsc_set_error(EFFSC_INVALID_ARG, "transcript %zu: wrong field or kind", i);
    }
    const size_t rows = row_off[n];
    if (rows && !round_polys) return effsc_set_error(EFFSC_INVALID_ARG, "round_polys is NULL");
    std::vector<u64> polys(rows * nw * 3, 0);
    for (size_t e = 0; e < rows * nw; e++)
        for (int c = 0; c < field; c++) polys[3 * e + c] = round_polys[e * field + c] % 0xFFFFFFFF00000001ULL;
    int rc = EFFSC_OK;
    u64 *d_claimed = nullptr, *d_polys = nullptr, *d_rows = nullptr, *d_ch = nullptr, *d_fin = nullptr;
    u32* d_rounds = nullptr;
    DevTranscript* d_tx = nullptr;
    uint8_t* d_hook = nullptr;
    std::vector<u64> ch, fin(3 * n);
    VCK(cudaMallocAsync((void**)&d_claimed, claimed.size() * 8, s));
    VCK(cudaMallocAsync((void**)&d_polys, std::max<size_t>(1, polys.size()) * 8, s));
    VCK(cudaMallocAsync((void**)&d_rows, row_off.size() * 8, s));
    VCK(cudaMallocAsync((void**)&d_rounds, n * 4, s));
    VCK(cudaMallocAsync((void**)&d_tx, n * sizeof(DevTranscript), s));
    VCK(cudaMallocAsync((void**)&d_fin, fin.size() * 8, s));
    if (challenges) VCK(cudaMallocAsync((void**)&d_ch, std::max<size_t>(1, rows) * 3 * 8, s));
    if (hook_len) VCK(cudaMallocAsync((void**)&d_hook, hook_len, s));
    VCK(cudaMemcpyAsync(d_claimed, claimed.data(), claimed.size() * 8, cudaMemcpyHostToDevice, s));
    if (!polys.empty()) VCK(cudaMemcpyAsync(d_polys, polys.data(), polys.size() * 8, cudaMemcpyHostToDevice, s));
    VCK(cudaMemcpyAsync(d_rows, row_off.data(), row_off.size() * 8, cudaMemcpyHostToDevice, s));
    VCK(cudaMemcpyAsync(d_rounds, num_rounds, n * 4, cudaMemcpyHostToDevice, s));
    VCK(cudaMemcpyAsync(d_tx, tx.data(), n * sizeof(DevTranscript), cudaMemcpyHostToDevice, s));
    if (hook_len) VCK(cudaMemcpyAsync(d_hook, hook, hook_len, cudaMemcpyHostToDevice, s));
    {
        VerifyArgs va;
        va.claimed = d_claimed; va.polys = d_polys; va.row_off = d_rows; va.rounds = d_rounds; va.tx = d_tx;
        va.hook = d_hook; va.hook_len = (u32)hook_len; va.degree = (u32)degree; va.n = (u32)n;
        va.challenges = d_ch; va.finals = d_fin;
        k_verify_batch<<<(unsigned)((n + 3) / 4), 128, 0, s>>>(va);
        effsc_internal_add_launches(1);
        VCK(cudaGetLastError());
    }
    VCK(cudaMemcpyAsync(fin.data(), d_fin, fin.size() * 8, cudaMemcpyDeviceToHost, s));
    if (challenges) {
        ch.resize(std::max<size_t>(1, rows) * 3);
        VCK(cudaMemcpyAsync(ch.data(), d_ch, ch.size() * 8, cudaMemcpyDeviceToHost, s));
    }
    VCK(cudaStreamSynchronize(s));
    for (size_t i = 0; i < n; i++)
        for (int c = 0; c < field; c++) final_claims[i * field + c] = fin[3 * i + c];
    if (challenges)
        for (size_t r = 0; r < rows; r++)
            for (int c = 0; c < field; c++) challenges[r * field + c] = ch[3 * r + c];
done:
    for (void* p : {(void*)d_claimed, (void*)d_polys, (void*)d_rows, (void*)d_rounds, (void*)d_tx, (void*)d_fin,
                    (void*)d_ch, (void*)d_hook})
        if (p) cudaFreeAsync(p, s);
    return rc;
}
