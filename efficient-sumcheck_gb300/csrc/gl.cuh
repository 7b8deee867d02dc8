// gl.cuh -- Goldilocks (p = 2^64 - 2^32 + 1) base field and its cubic extension
// Fp3 = Fp[X]/(X^3 - W) on sm_103a.
//
// Values live in HBM in canonical form (0 <= x < p).  The reference crate keeps
// arkworks Montgomery residues (src/field.rs:314-375); the boundary converts.
// W is the canonical value of the crate's F64Ext3 non-residue F64::from_raw(7)
// (src/tests/fields.rs:73-100), i.e. 7 * 2^-64 mod p = -7 * 2^32 mod p.
//
// Sums of products are accumulated lazily in 160-bit accumulators of five
// 32-bit limbs (32x32-bit multiply-add chains with carry) and reduced once
// with 2^64 = 2^32 - 1 and 2^96 = -1 (mod p).  Single products outside the hot
// loops use a 128-bit product and the same reduction.
#pragma once
#include <cstdint>

#include "gl_w.h"

typedef unsigned long long u64;
typedef unsigned int u32;

#define GL_P 0xFFFFFFFF00000001ULL
#define GL_EPS 0x00000000FFFFFFFFULL
#define GL_W 0xFFFFFFF800000001ULL

__device__ __forceinline__ u64 gl_add(u64 a, u64 b) {
    u64 s = a + b;
    if (s < a) return s + GL_EPS;            // carry: 2^64 = eps; result already < p
    return s >= GL_P ? s - GL_P : s;
}
// a - b for canonical a, b; on a borrow subtract 2^32 - 1 (i.e. add p mod 2^64).
__device__ __forceinline__ u64 gl_sub(u64 a, u64 b) {
    u32 d0, d1;
    asm("{\n\t.reg .u32 m;\n\t"
        "sub.cc.u32 %0, %2, %4;\n\t"
        "subc.cc.u32 %1, %3, %5;\n\t"
        "subc.u32 m, 0, 0;\n\t"
        "sub.cc.u32 %0, %0, m;\n\t"
        "subc.u32 %1, %1, 0;\n\t}"
        : "=r"(d0), "=r"(d1)
        : "r"((u32)a), "r"((u32)(a >> 32)), "r"((u32)b), "r"((u32)(b >> 32)));
    return ((u64)d1 << 32) | d0;
}
__device__ __forceinline__ u64 gl_neg(u64 a) { return a ? GL_P - a : 0; }

// (hi:lo) mod p, canonical
__device__ __forceinline__ u64 gl_reduce128(u64 lo, u64 hi) {
    u64 hh = hi >> 32, hl = hi & GL_EPS;
    u64 t0 = lo - hh;
    if (lo < hh) t0 -= GL_EPS;
    u64 t1 = (hl << 32) - hl;
    u64 t2 = t0 + t1;
    if (t2 < t1) t2 += GL_EPS;
    return t2 >= GL_P ? t2 - GL_P : t2;
}
__device__ __forceinline__ void gl_mul128(u64 a, u64 b, u64& lo, u64& hi) {
    lo = a * b;
    hi = __umul64hi(a, b);
}
__device__ __forceinline__ u64 gl_mul(u64 a, u64 b) {
    u64 lo, hi;
    gl_mul128(a, b, lo, hi);
    return gl_reduce128(lo, hi);
}

// ---- lazy 160-bit accumulator -------------------------------------------------
// Five 32-bit limbs c0..c4 (value c0 + c1 2^32 + ... + c4 2^128).  A product is
// added with a chain of eight 32-bit multiply-adds with carry (mad.lo.cc /
// madc.hi.cc), so no 128-bit intermediate and no separate carry handling.
__device__ __forceinline__ u32 lo32(u64 x) { return (u32)x; }
__device__ __forceinline__ u32 hi32(u64 x) { return (u32)(x >> 32); }
__device__ __forceinline__ u64 mk64(u32 lo, u32 hi) { return ((u64)hi << 32) | lo; }

struct Acc {
    u32 c0, c1, c2, c3, c4;
};
__device__ __forceinline__ Acc acc_zero() { Acc a; a.c0 = a.c1 = a.c2 = a.c3 = a.c4 = 0; return a; }
__device__ __forceinline__ Acc acc_from(u64 v) { Acc a; a.c0 = lo32(v); a.c1 = hi32(v); a.c2 = a.c3 = a.c4 = 0; return a; }
__device__ __forceinline__ void acc_mac(Acc& s, u64 x, u64 y) {
    const u32 x0 = lo32(x), x1 = hi32(x), y0 = lo32(y), y1 = hi32(y);
    asm("mad.lo.cc.u32 %0, %5, %7, %0;\n\t"
        "madc.hi.cc.u32 %1, %5, %7, %1;\n\t"
        "madc.lo.cc.u32 %2, %6, %8, %2;\n\t"
        "madc.hi.cc.u32 %3, %6, %8, %3;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %1, %5, %8, %1;\n\t"
        "madc.hi.cc.u32 %2, %5, %8, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %1, %6, %7, %1;\n\t"
        "madc.hi.cc.u32 %2, %6, %7, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;"
        : "+r"(s.c0), "+r"(s.c1), "+r"(s.c2), "+r"(s.c3), "+r"(s.c4)
        : "r"(x0), "r"(x1), "r"(y0), "r"(y1));
}
__device__ __forceinline__ void acc_add64(Acc& s, u64 v) {
    asm("add.cc.u32 %0, %0, %5;\n\t"
        "addc.cc.u32 %1, %1, %6;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;"
        : "+r"(s.c0), "+r"(s.c1), "+r"(s.c2), "+r"(s.c3), "+r"(s.c4)
        : "r"(lo32(v)), "r"(hi32(v)));
}
// Canonical value mod p.  With B = 2^32: B^2 = B - 1 and B^3 = -1 (mod p), so
//   x = (c1:c0) - (c4:c3) + c2 (B - 1).
// The 64-bit subtraction and addition leave a net carry cm in {-1, 0, 1}
// worth cm * 2^64 = cm (B - 1); adding that back can underflow only when
// cm = -1, and then once more by B - 1.  A final conditional subtraction of p
// gives the canonical residue.
__device__ __forceinline__ u64 acc_reduce(const Acc& s) {
    u32 r0, r1;
    asm("{\n\t"
        ".reg .u32 t0, t1, bm, e0, e1, cm, sx, f0, f1, cc2, nf, d, v0, v1, ge;\n\t"
        ".reg .pred pge;\n\t"
        "sub.cc.u32 t0, %2, %5;\n\t"
        "subc.cc.u32 t1, %3, %6;\n\t"
        "subc.u32 bm, 0, 0;\n\t"
        "sub.cc.u32 e0, 0, %4;\n\t"
        "subc.u32 e1, %4, 0;\n\t"
        "add.cc.u32 t0, t0, e0;\n\t"
        "addc.cc.u32 t1, t1, e1;\n\t"
        "addc.u32 cm, bm, 0;\n\t"
        "shr.s32 sx, cm, 31;\n\t"
        "sub.cc.u32 f0, 0, cm;\n\t"
        "subc.u32 f1, cm, sx;\n\t"
        "add.cc.u32 t0, t0, f0;\n\t"
        "addc.cc.u32 t1, t1, f1;\n\t"
        "addc.u32 cc2, 0, 0;\n\t"
        "shr.u32 nf, cm, 31;\n\t"
        "sub.u32 d, cc2, nf;\n\t"
        "sub.cc.u32 t0, t0, d;\n\t"
        "subc.u32 t1, t1, 0;\n\t"
        "add.cc.u32 v0, t0, 0xFFFFFFFF;\n\t"
        "addc.cc.u32 v1, t1, 0;\n\t"
        "addc.u32 ge, 0, 0;\n\t"
        "setp.ne.u32 pge, ge, 0;\n\t"
        "selp.b32 %0, v0, t0, pge;\n\t"
        "selp.b32 %1, v1, t1, pge;\n\t"
        "}"
        : "=r"(r0), "=r"(r1)
        : "r"(s.c0), "r"(s.c1), "r"(s.c2), "r"(s.c3), "r"(s.c4));
    return mk64(r0, r1);
}

// ---- split accumulator --------------------------------------------------------
// The same sum kept as a 160-bit part s (the products x0 y0 + x1 y1 2^64) and
// a 96-bit part m (the middle products x0 y1 + x1 y0, worth m 2^32): a
// product costs 8 multiply-adds and 3 carry adds (acc_mac: 8 and 5) in two
// independent carry chains, for 3 more registers.
struct AccS {
    u32 s0, s1, s2, s3, s4, m0, m1, m2;
};
__device__ __forceinline__ AccS accs_zero() { AccS a; a.s0 = a.s1 = a.s2 = a.s3 = a.s4 = a.m0 = a.m1 = a.m2 = 0; return a; }
__device__ __forceinline__ AccS accs_from(u64 v) { AccS a = accs_zero(); a.s0 = lo32(v); a.s1 = hi32(v); return a; }
__device__ __forceinline__ void accs_mac(AccS& s, u64 x, u64 y) {
    const u32 x0 = lo32(x), x1 = hi32(x), y0 = lo32(y), y1 = hi32(y);
    asm("mad.lo.cc.u32 %0, %8, %10, %0;\n\t"
        "madc.hi.cc.u32 %1, %8, %10, %1;\n\t"
        "madc.lo.cc.u32 %2, %9, %11, %2;\n\t"
        "madc.hi.cc.u32 %3, %9, %11, %3;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %5, %8, %11, %5;\n\t"
        "madc.hi.cc.u32 %6, %8, %11, %6;\n\t"
        "addc.u32 %7, %7, 0;\n\t"
        "mad.lo.cc.u32 %5, %9, %10, %5;\n\t"
        "madc.hi.cc.u32 %6, %9, %10, %6;\n\t"
        "addc.u32 %7, %7, 0;"
        : "+r"(s.s0), "+r"(s.s1), "+r"(s.s2), "+r"(s.s3), "+r"(s.s4), "+r"(s.m0), "+r"(s.m1), "+r"(s.m2)
        : "r"(x0), "r"(x1), "r"(y0), "r"(y1));
}
// s + m 2^32 as one 160-bit accumulator (below 2^160 for fewer than 2^31 products).
__device__ __forceinline__ Acc accs_join(const AccS& s) {
    Acc a;
    a.c0 = s.s0; a.c1 = s.s1; a.c2 = s.s2; a.c3 = s.s3; a.c4 = s.s4;
    asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\taddc.cc.u32 %2, %2, %6;\n\taddc.u32 %3, %3, 0;"
        : "+r"(a.c1), "+r"(a.c2), "+r"(a.c3), "+r"(a.c4) : "r"(s.m0), "r"(s.m1), "r"(s.m2));
    return a;
}
__device__ __forceinline__ u64 accs_reduce(const AccS& s) { return acc_reduce(accs_join(s)); }

// The two accumulator forms behind one interface: FORM 0 = Acc (5 registers,
// for sums that stay live across a loop), FORM 1 = AccS (8 registers, two
// carry chains; measured 7% faster in the Fp3 folds, slower where ten
// accumulators stay live).
template <int FORM> struct AccF;
template <> struct AccF<0> {
    Acc a;
    __device__ __forceinline__ void zero() { a = acc_zero(); }
    __device__ __forceinline__ void from(u64 v) { a = acc_from(v); }
    __device__ __forceinline__ void mac(u64 x, u64 y) { acc_mac(a, x, y); }
    __device__ __forceinline__ u64 reduce() const { return acc_reduce(a); }
};
template <> struct AccF<1> {
    AccS a;
    __device__ __forceinline__ void zero() { a = accs_zero(); }
    __device__ __forceinline__ void from(u64 v) { a = accs_from(v); }
    __device__ __forceinline__ void mac(u64 x, u64 y) { accs_mac(a, x, y); }
    __device__ __forceinline__ u64 reduce() const { return accs_reduce(a); }
};
// Short sums reduced right away (a fold's output component) use the split form.
constexpr int FOLD_FORM = 1;

// ---- Fp3 ---------------------------------------------------------------------
// E == false: only c0 is meaningful (a base-field value embedded as (c0,0,0)).
struct F3 {
    u64 c0, c1, c2;
};
__device__ __forceinline__ F3 f3_zero() { F3 r; r.c0 = r.c1 = r.c2 = 0; return r; }
__device__ __forceinline__ F3 f3_make(u64 a, u64 b, u64 c) { F3 r; r.c0 = a; r.c1 = b; r.c2 = c; return r; }

template <bool E>
__device__ __forceinline__ F3 f3_add(const F3& a, const F3& b) {
    F3 r;
    r.c0 = gl_add(a.c0, b.c0);
    if (E) { r.c1 = gl_add(a.c1, b.c1); r.c2 = gl_add(a.c2, b.c2); } else { r.c1 = r.c2 = 0; }
    return r;
}
template <bool E>
__device__ __forceinline__ F3 f3_sub(const F3& a, const F3& b) {
    F3 r;
    r.c0 = gl_sub(a.c0, b.c0);
    if (E) { r.c1 = gl_sub(a.c1, b.c1); r.c2 = gl_sub(a.c2, b.c2); } else { r.c1 = r.c2 = 0; }
    return r;
}
// Mixed add where the second operand may be base (EB false).
template <bool EA, bool EB>
__device__ __forceinline__ F3 f3_add_mixed(const F3& a, const F3& b) {
    F3 r;
    r.c0 = gl_add(a.c0, b.c0);
    if (EA && EB) { r.c1 = gl_add(a.c1, b.c1); r.c2 = gl_add(a.c2, b.c2); }
    else if (EA) { r.c1 = a.c1; r.c2 = a.c2; }
    else if (EB) { r.c1 = b.c1; r.c2 = b.c2; }
    else { r.c1 = r.c2 = 0; }
    return r;
}

// A multiplier prepared for repeated use: (m0, m1, m2, W*m1, W*m2).
struct Mul3 {
    u64 m0, m1, m2, w1, w2;
};
template <bool E>
__device__ __forceinline__ Mul3 mul3_prepare(const F3& m) {
    Mul3 r;
    r.m0 = m.c0;
    if (E) { r.m1 = m.c1; r.m2 = m.c2; r.w1 = gl_mul_w(m.c1); r.w2 = gl_mul_w(m.c2); }
    else { r.m1 = r.m2 = r.w1 = r.w2 = 0; }
    return r;
}
// x * m (+ add), reduced.  EX: x is Fp3; EM: m is Fp3; EADD: add is Fp3.
// (d0 + d1 X + d2 X^2)(m0 + m1 X + m2 X^2) mod X^3 - W:
//   c0 = d0 m0 + d1 (W m2) + d2 (W m1)
//   c1 = d0 m1 + d1 m0 + d2 (W m2)
//   c2 = d0 m2 + d1 m1 + d2 m0
template <bool EX, bool EM, bool EADD, bool HAS_ADD>
__device__ __forceinline__ F3 f3_mul_add(const F3& x, const Mul3& m, const F3& add) {
    F3 r;
    AccF<FOLD_FORM> a0, a1, a2;
    a0.from(HAS_ADD ? add.c0 : 0);
    if (!EX && !EM) {
        a0.mac(x.c0, m.m0);
        r.c0 = a0.reduce();
        if (HAS_ADD && EADD) { r.c1 = add.c1; r.c2 = add.c2; } else { r.c1 = r.c2 = 0; }
        return r;
    }
    a1.from(HAS_ADD && EADD ? add.c1 : 0);
    a2.from(HAS_ADD && EADD ? add.c2 : 0);
    if (EX != EM) {
        // one side base: three independent products
        u64 b = EX ? m.m0 : x.c0;
        a0.mac(EX ? x.c0 : m.m0, b);
        a1.mac(EX ? x.c1 : m.m1, b);
        a2.mac(EX ? x.c2 : m.m2, b);
    } else {
        a0.mac(x.c0, m.m0); a0.mac(x.c1, m.w2); a0.mac(x.c2, m.w1);
        a1.mac(x.c0, m.m1); a1.mac(x.c1, m.m0); a1.mac(x.c2, m.w2);
        a2.mac(x.c0, m.m2); a2.mac(x.c1, m.m1); a2.mac(x.c2, m.m0);
    }
    r.c0 = a0.reduce();
    r.c1 = a1.reduce();
    r.c2 = a2.reduce();
    return r;
}
template <bool EA, bool EB>
__device__ __forceinline__ F3 f3_mul(const F3& a, const F3& b) {
    Mul3 m = mul3_prepare<EB>(b);
    return f3_mul_add<EA, EB, false, false>(a, m, f3_zero());
}

// Lazy sum of products: accumulates sum a*b with a in F<EA>, b in F<EB>.
template <bool EA, bool EB, int FORM = 0>
struct ProdAcc {
    AccF<FORM> s0, s0w, s1, s1w, s2;
    __device__ __forceinline__ void init() { s0.zero(); s0w.zero(); s1.zero(); s1w.zero(); s2.zero(); }
    __device__ __forceinline__ void mac(const F3& a, const F3& b) {
        s0.mac(a.c0, b.c0);
        if (EA && EB) {
            s0w.mac(a.c1, b.c2); s0w.mac(a.c2, b.c1);
            s1.mac(a.c0, b.c1); s1.mac(a.c1, b.c0);
            s1w.mac(a.c2, b.c2);
            s2.mac(a.c0, b.c2); s2.mac(a.c1, b.c1); s2.mac(a.c2, b.c0);
        } else if (EA) {
            s1.mac(a.c1, b.c0); s2.mac(a.c2, b.c0);
        } else if (EB) {
            s1.mac(a.c0, b.c1); s2.mac(a.c0, b.c2);
        }
    }
    __device__ __forceinline__ F3 result() const {
        F3 r;
        r.c0 = s0.reduce();
        if (EA || EB) {
            r.c1 = s1.reduce();
            r.c2 = s2.reduce();
            if (EA && EB) {
                r.c0 = gl_add(r.c0, gl_mul_w(s0w.reduce()));
                r.c1 = gl_add(r.c1, gl_mul_w(s1w.reduce()));
            }
        } else {
            r.c1 = r.c2 = 0;
        }
        return r;
    }
};
// Lazy sum of products (ab) c with both Fp3: c prepared with W per product
// (two multiplications by W, no general product) so that three accumulators
// hold the sum instead of five; the same value as ProdAcc<true, true>.
template <bool EA, bool EB>
struct PointAcc {
    ProdAcc<EA, EB> p;
    __device__ __forceinline__ void init() { p.init(); }
    __device__ __forceinline__ void mac(const F3& a, const F3& b) { p.mac(a, b); }
    __device__ __forceinline__ F3 result() const { return p.result(); }
};
template <>
struct PointAcc<true, true> {
    AccF<0> s0, s1, s2;
    __device__ __forceinline__ void init() { s0.zero(); s1.zero(); s2.zero(); }
    __device__ __forceinline__ void mac(const F3& a, const F3& b) {
        const Mul3 m = mul3_prepare<true>(b);
        s0.mac(a.c0, m.m0); s0.mac(a.c1, m.w2); s0.mac(a.c2, m.w1);
        s1.mac(a.c0, m.m1); s1.mac(a.c1, m.m0); s1.mac(a.c2, m.w2);
        s2.mac(a.c0, m.m2); s2.mac(a.c1, m.m1); s2.mac(a.c2, m.m0);
    }
    __device__ __forceinline__ F3 result() const { return f3_make(s0.reduce(), s1.reduce(), s2.reduce()); }
};

// Lazy sum of field elements.
template <bool E>
struct SumAcc {
    Acc s0, s1, s2;
    __device__ __forceinline__ void init() { s0 = s1 = s2 = acc_zero(); }
    __device__ __forceinline__ void add(const F3& a) {
        acc_add64(s0, a.c0);
        if (E) { acc_add64(s1, a.c1); acc_add64(s2, a.c2); }
    }
    __device__ __forceinline__ F3 result() const {
        F3 r;
        r.c0 = acc_reduce(s0);
        if (E) { r.c1 = acc_reduce(s1); r.c2 = acc_reduce(s2); } else { r.c1 = r.c2 = 0; }
        return r;
    }
};

// Fold: lo + (hi - lo) * r  with r prepared as Mul3.
template <bool EIN, bool ECH>
__device__ __forceinline__ F3 f3_fold(const F3& lo, const F3& hi, const Mul3& r) {
    F3 d = f3_sub<EIN>(hi, lo);
    return f3_mul_add<EIN, ECH, EIN, true>(d, r, lo);
}
