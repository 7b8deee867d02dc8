// keccak.cuh -- the Fiat-Shamir transcript on the device.
//
// Keccak-f[1600] (FIPS 202) with one 64-bit lane per thread of a warp (lanes
// 25..31 shadow lanes and are ignored), used as a duplex sponge with a
// 136-byte rate.  The host transcript (runtime.cu) and the CPU oracle
// implement the same byte-exact construction:
//   * absorb(bytes): after a squeeze, restart at byte 0 of the rate without a
//     permutation (duplex); permute whenever a byte must go past the rate;
//     XOR bytes into the state little-endian;
//   * squeeze(n): on the first squeeze after absorbing, XOR 0x06 at the
//     current position and 0x80 at byte 135, permute, restart at byte 0;
//     permute whenever a byte must come from past the rate;
//   * an Fp element is sent as 8 LE bytes, an Fp3 element as 3 x 8 LE bytes;
//   * a challenge component is 16 squeezed LE bytes reduced mod p.
#pragma once
#include "gl.cuh"

#define TX_RATE 136

// Layout shared with the host (runtime.cu): 216 bytes.
struct DevTranscript {
    u64 st[25];
    u32 pos;
    u32 squeezing;
    u32 deg;
    u32 reserved;
};

static __constant__ u64 c_keccak_rc[24] = {
    0x0000000000000001ULL, 0x0000000000008082ULL, 0x800000000000808AULL, 0x8000000080008000ULL,
    0x000000000000808BULL, 0x0000000080000001ULL, 0x8000000080008081ULL, 0x8000000000008009ULL,
    0x000000000000008AULL, 0x0000000000000088ULL, 0x0000000080008009ULL, 0x000000008000000AULL,
    0x000000008000808BULL, 0x800000000000008BULL, 0x8000000000008089ULL, 0x8000000000008003ULL,
    0x8000000000008002ULL, 0x8000000000000080ULL, 0x000000000000800AULL, 0x800000008000000AULL,
    0x8000000080008081ULL, 0x8000000000008080ULL, 0x0000000080000001ULL, 0x8000000080008008ULL};

// rotation offsets (rho), indexed by lane x + 5y
static __constant__ int c_keccak_rot[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43,
                                            25, 39, 41, 45, 15, 21, 8, 18, 2, 61, 56, 14};

__device__ __forceinline__ u64 shfl64(u64 v, int src) {
    u32 lo = __shfl_sync(0xffffffffu, (u32)v, src);
    u32 hi = __shfl_sync(0xffffffffu, (u32)(v >> 32), src);
    return ((u64)hi << 32) | lo;
}
__device__ __forceinline__ u64 rotl64d(u64 x, int r) {
    return (x << r) | (x >> ((64 - r) & 63));
}

// One Keccak-f[1600] permutation; lane i (< 25) holds lane A[i], i = x + 5y.
// The round is bound by shuffle latency and count (one warp, nothing to
// overlap with), so each step uses as few as it can: theta's column parities
// by a tree over the rows (y, y+1; then +2 rows; then row 4: three 64-bit
// shuffles, the parity of column x lands in lane x), then C[x-1] and C[x+1];
// pi and chi take B[x, y], B[x+1, y] and B[x+2, y] straight from the lanes
// that rho-rotate into them.  Eight 64-bit shuffles per round.
static __device__ __noinline__ void keccak_f_warp(u64& a, int lane) {
    const int i = lane < 25 ? lane : 0;
    const int x = i % 5, y = i / 5;
    const int my_rot = c_keccak_rot[i];
    // pi: B[X, Y] = rho(A[x, y]) with X = y, Y = 2x + 3y; the source of lane
    // (X, Y) is x = (X + 3Y) mod 5, y = X.
    const int xp1 = (x + 1) % 5, xp2 = (x + 2) % 5, xm1 = (x + 4) % 5;
    const int src0 = ((x + 3 * y) % 5) + 5 * x;
    const int src1 = ((xp1 + 3 * y) % 5) + 5 * xp1;
    const int src2 = ((xp2 + 3 * y) % 5) + 5 * xp2;
    const int l5 = min(i + 5, 31), l10 = min(i + 10, 31), l20 = min(i + 20, 31);
#pragma unroll 1
    for (int round = 0; round < 24; round++) {
        u64 v = a ^ shfl64(a, l5);           // rows y, y+1
        const u64 a20 = shfl64(a, l20);      // row y+4 (used by lanes 0..4)
        v ^= shfl64(v, l10);                 // rows y..y+3
        v ^= a20;                            // lanes 0..4: C[x]
        const u64 cm = shfl64(v, xm1), cp = shfl64(v, xp1);
        a ^= cm ^ rotl64d(cp, 1);
        const u64 r = rotl64d(a, my_rot);
        const u64 b = shfl64(r, src0), b1 = shfl64(r, src1), b2 = shfl64(r, src2);
        a = b ^ (~b1 & b2);
        if (lane == 0) a ^= c_keccak_rc[round];
    }
    if (lane >= 25) a = 0;
}

// Transcript state held by one warp: lane state word, byte position, mode.
struct WarpTx {
    u64 a;
    u32 pos;
    u32 squeezing;
    u32 deg;
};

__device__ __forceinline__ WarpTx tx_load(const DevTranscript* t, int lane) {
    WarpTx w;
    w.a = lane < 25 ? t->st[lane] : 0;
    w.pos = t->pos;
    w.squeezing = t->squeezing;
    w.deg = t->deg;
    return w;
}
__device__ __forceinline__ void tx_store(DevTranscript* t, const WarpTx& w, int lane) {
    if (lane < 25) t->st[lane] = w.a;
    if (lane == 0) { t->pos = w.pos; t->squeezing = w.squeezing; t->deg = w.deg; }
}

// XOR `len` bytes (read through `get(k)`, k in [0,len)) into the rate.
template <class Get>
__device__ __forceinline__ void tx_absorb(WarpTx& w, int lane, u32 len, Get get) {
    if (w.squeezing) { w.pos = 0; w.squeezing = 0; }
    u32 done = 0;
    while (done < len) {
        if (w.pos == TX_RATE) { keccak_f_warp(w.a, lane); w.pos = 0; }
        u32 chunk = min(len - done, (u32)TX_RATE - w.pos);
        if (lane < TX_RATE / 8) {
            u64 x = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                u32 g = 8 * lane + k;
                if (g >= w.pos && g < w.pos + chunk) x |= (u64)get(done + (g - w.pos)) << (8 * k);
            }
            w.a ^= x;
        }
        w.pos += chunk;
        done += chunk;
    }
}
// Squeeze `len` bytes, handing byte k to `put(k, byte)` on the owning lane.
template <class Put>
__device__ __forceinline__ void tx_squeeze(WarpTx& w, int lane, u32 len, Put put) {
    if (!w.squeezing) {
        if (w.pos == TX_RATE) { keccak_f_warp(w.a, lane); w.pos = 0; }
        if (lane == (int)(w.pos >> 3)) w.a ^= (u64)0x06 << (8 * (w.pos & 7));
        if (lane == (TX_RATE - 1) / 8) w.a ^= (u64)0x80 << (8 * ((TX_RATE - 1) & 7));
        keccak_f_warp(w.a, lane);
        w.pos = 0;
        w.squeezing = 1;
    }
    u32 done = 0;
    while (done < len) {
        if (w.pos == TX_RATE) { keccak_f_warp(w.a, lane); w.pos = 0; }
        u32 chunk = min(len - done, (u32)TX_RATE - w.pos);
        if (lane < TX_RATE / 8) {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                u32 g = 8 * lane + k;
                if (g >= w.pos && g < w.pos + chunk) put(done + (g - w.pos), (uint8_t)(w.a >> (8 * k)));
            }
        }
        w.pos += chunk;
        done += chunk;
    }
}

// Word-aligned forms of absorb / squeeze (w.pos % 8 == 0): the same bytes in
// the same order, one 64-bit word per lane instead of one byte per step.
template <class GetW>
__device__ __forceinline__ void tx_absorb_words(WarpTx& w, int lane, u32 nwords, GetW getw) {
    if (w.squeezing) { w.pos = 0; w.squeezing = 0; }
    u32 done = 0;
    while (done < nwords) {
        if (w.pos == TX_RATE) { keccak_f_warp(w.a, lane); w.pos = 0; }
        const u32 p8 = w.pos >> 3;
        const u32 chunk = min(nwords - done, (u32)(TX_RATE / 8) - p8);
        if ((u32)lane >= p8 && (u32)lane < p8 + chunk) w.a ^= getw(done + (u32)lane - p8);
        w.pos += 8 * chunk;
        done += chunk;
    }
}
template <class PutW>
__device__ __forceinline__ void tx_squeeze_words(WarpTx& w, int lane, u32 nwords, PutW putw) {
    if (!w.squeezing) {
        if (w.pos == TX_RATE) { keccak_f_warp(w.a, lane); w.pos = 0; }
        if (lane == (int)(w.pos >> 3)) w.a ^= (u64)0x06 << (8 * (w.pos & 7));
        if (lane == (TX_RATE - 1) / 8) w.a ^= (u64)0x80 << (8 * ((TX_RATE - 1) & 7));
        keccak_f_warp(w.a, lane);
        w.pos = 0;
        w.squeezing = 1;
    }
    u32 done = 0;
    while (done < nwords) {
        if (w.pos == TX_RATE) { keccak_f_warp(w.a, lane); w.pos = 0; }
        const u32 p8 = w.pos >> 3;
        const u32 chunk = min(nwords - done, (u32)(TX_RATE / 8) - p8);
        if ((u32)lane >= p8 && (u32)lane < p8 + chunk) putw(done + (u32)lane - p8, w.a);
        w.pos += 8 * chunk;
        done += chunk;
    }
}

// Absorb `n` field elements (deg components each) from shared memory `v`
// (layout: element e component c at v[3e + c]).
__device__ __forceinline__ void tx_send_elems(WarpTx& w, int lane, const u64* v, int n) {
    const u32 deg = w.deg;
    if ((w.pos & 7) == 0 || w.squeezing) {
        tx_absorb_words(w, lane, (u32)n * deg, [&](u32 word) -> u64 {
            const u32 e = deg == 3 ? word / 3 : word, c = deg == 3 ? word % 3 : 0;
            return v[3 * e + c];
        });
        return;
    }
    tx_absorb(w, lane, (u32)n * deg * 8, [&](u32 k) -> uint8_t {
        u32 word = k >> 3, e = word / deg, c = word % deg;
        return (uint8_t)(v[3 * e + c] >> (8 * (k & 7)));
    });
}
// Squeeze one challenge into shared memory `out` (3 words; unused set to 0).
// `scratch` is 48 bytes of 8-byte aligned shared memory.
__device__ __forceinline__ void tx_challenge(WarpTx& w, int lane, u64* out, uint8_t* scratch) {
    const u32 deg = w.deg;
    // the first squeeze after absorbing pads and restarts at byte 0, so the
    // word form applies whenever the rate position is a multiple of 8
    if (!w.squeezing || (w.pos & 7) == 0) {
        u64* sw = (u64*)scratch;
        tx_squeeze_words(w, lane, 2 * deg, [&](u32 k, u64 v) { sw[k] = v; });
    } else {
        tx_squeeze(w, lane, 16 * deg, [&](u32 k, uint8_t b) { scratch[k] = b; });
    }
    __syncwarp();
    if (lane < 3) {
        u64 r = 0;
        if ((u32)lane < deg) {
            const u64* sw = (const u64*)scratch;   // little-endian bytes
            r = gl_reduce128(sw[2 * lane], sw[2 * lane + 1]);
        }
        out[lane] = r;
    }
    __syncwarp();
}
