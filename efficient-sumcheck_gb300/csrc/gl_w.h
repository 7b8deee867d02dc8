// gl_w.h -- multiplication by the Fp3 non-residue W without a general product.
//
// F64Ext3 is Fp[X]/(X^3 - W) with W = 0xFFFFFFF800000001 = 2^64 - 2^35 + 1
// (the crate's from_raw(7): 7 * 2^-64 mod p).  Since 2^64 = 2^32 - 1 (mod p),
// W = 2^32 - 1 - 2^35 + 1 = -7 * 2^32 (mod p), so W x is a shift, a
// subtraction and the folding of 2^64 and 2^96 (2^96 = -1), with no 64 x 64
// product:
//   y = 7x = hi 2^64 + lo            (hi <= 6)
//   y 2^32 = lo 2^32 + hi 2^96 = (a + b) 2^32 - b - hi   (lo = a + b 2^32)
//   (a + b) 2^32 = tl 2^32 + th (2^32 - 1)              (a + b = tl + th 2^32)
//   W x = -(y 2^32) = (b + hi) - (tl 2^32 + th (2^32 - 1))
// Plain 64-bit C, shared by the kernels and the host tests.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GLW_FN __host__ __device__ __forceinline__
#else
#define GLW_FN static inline
#endif

GLW_FN uint64_t gl_mul_w(uint64_t x) {
    const uint64_t P = 0xFFFFFFFF00000001ULL;
    const uint64_t x8 = x << 3, h8 = x >> 61;
    const uint64_t lo = x8 - x, hi = h8 - (x8 < x ? 1u : 0u);   // 7x
    const uint64_t a = lo & 0xFFFFFFFFULL, b = lo >> 32;
    const uint64_t t = a + b;                                    // < 2^33
    uint64_t v = ((t & 0xFFFFFFFFULL) << 32) + (t >> 32) * 0xFFFFFFFFULL;   // <= 2^64 - 1
    if (v >= P) v -= P;
    const uint64_t u = b + hi;                                   // < 2^32 + 7 < p
    return u >= v ? u - v : u - v + P;
}
