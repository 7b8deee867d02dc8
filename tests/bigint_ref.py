"""Independent pure-Python (big-integer) restatement of the reference provers.

Used only by the CPU tests, on small inputs, to pin the C oracle: every value
here is computed with Python integers and ``%``, the cubic extension by
polynomial multiplication reduced with X^3 = W, and W derived from the crate's
``F64::from_raw(7)`` (a Montgomery raw value) as ``7 * 2^-64 mod p``
(reference src/tests/fields.rs:73-100).  The prover bodies follow the
reference's *unfused* test provers (tests/inner_product_sumcheck.rs:212-296,
tests/multilinear_sumcheck.rs) and the provers in src/provers/.
"""
P = (1 << 64) - (1 << 32) + 1
R_INV = pow(1 << 64, -1, P)
W = 7 * R_INV % P

ZERO = (0, 0, 0)
ONE = (1, 0, 0)


def add(a, b):
    return tuple((x + y) % P for x, y in zip(a, b))


def sub(a, b):
    return tuple((x - y) % P for x, y in zip(a, b))


def mul(a, b):
    prod = [0] * 5
    for i in range(3):
        for j in range(3):
            prod[i + j] += a[i] * b[j]
    # X^3 = W, X^4 = W X
    c0 = prod[0] + W * prod[3]
    c1 = prod[1] + W * prod[4]
    c2 = prod[2]
    return (c0 % P, c1 % P, c2 % P)


def lift(x):
    return (int(x) % P, 0, 0)


def np2(n):
    p = 1
    while p < n:
        p <<= 1
    return p


def fold_msb_pad(v, w):
    """src/inner_product_sumcheck.rs:143-176 (and multilinear fold)."""
    n = len(v)
    if n <= 1:
        return list(v)
    half = np2(n) >> 1
    out = []
    for i in range(half):
        if i + half < n:
            out.append(add(v[i], mul(sub(v[i + half], v[i]), w)))
        else:
            out.append(mul(v[i], sub(ONE, w)))
    return out


def fold_msb_floor(v, c):
    n = len(v)
    if n <= 1:
        return list(v)
    half = n // 2
    return [add(v[k], mul(c, sub(v[k + half], v[k]))) for k in range(half)]


def fold_lsb(v, w):
    n = len(v)
    if n <= 1:
        return list(v)
    return [add(v[2 * i], mul(w, sub(v[2 * i + 1], v[2 * i]))) for i in range(n // 2)]


def ml_msb_compute(v):
    n = len(v)
    if n == 0:
        return ZERO, ZERO
    if n == 1:
        return v[0], ZERO
    half = np2(n) >> 1
    s0, s1 = ZERO, ZERO
    for i in range(half):
        s0 = add(s0, v[i])
        if i + half < n:
            s1 = add(s1, v[i + half])
    return s0, s1


def ml_lsb_compute(v):
    n = len(v)
    if n == 0:
        return ZERO, ZERO
    if n == 1:
        return v[0], ZERO
    s0, s1 = ZERO, ZERO
    for i in range(0, n, 2):
        s0 = add(s0, v[i])
        if i + 1 < n:
            s1 = add(s1, v[i + 1])
    return s0, s1


def ip_msb_compute(a, b):
    n = len(a)
    if n == 0:
        return ZERO, ZERO
    if n == 1:
        return mul(a[0], b[0]), ZERO
    half = np2(n) >> 1
    q0, qi = ZERO, ZERO
    for i in range(half):
        if i + half < n:
            q0 = add(q0, mul(a[i], b[i]))
            qi = add(qi, mul(sub(a[i + half], a[i]), sub(b[i + half], b[i])))
        else:
            t = mul(a[i], b[i])
            q0 = add(q0, t)
            qi = add(qi, t)
    return q0, qi


def ip_lsb_compute(a, b):
    n = len(a)
    if n == 0:
        return ZERO, ZERO
    if n == 1:
        return mul(a[0], b[0]), ZERO
    q0, qi = ZERO, ZERO
    for k in range(n // 2):
        ae, ao, be, bo = a[2 * k], a[2 * k + 1], b[2 * k], b[2 * k + 1]
        q0 = add(q0, mul(ae, be))
        qi = add(qi, mul(sub(ao, ae), sub(bo, be)))
    if n % 2:
        q0 = add(q0, mul(a[n - 1], b[n - 1]))
    return q0, qi


def product_coeffs(lo, hi):
    c = [ONE]
    for l, h in zip(lo, hi):
        d = sub(h, l)
        n = [ZERO] * (len(c) + 1)
        for j, cj in enumerate(c):
            n[j] = add(n[j], mul(cj, l))
            n[j + 1] = add(n[j + 1], mul(cj, d))
        c = n
    return c


def horner(c, x):
    r = c[-1]
    for ci in reversed(c[:-1]):
        r = add(mul(r, x), ci)
    return r


def build_eq(w):
    """src/provers/eq_factored.rs:217-239, MSB layout."""
    v = len(w)
    t = [ZERO] * (1 << v)
    t[0] = ONE
    for j, wj in enumerate(w):
        stride = 1 << (v - 1 - j)
        for b in range(1 << j):
            base = b * 2 * stride
            parent = t[base]
            t[base] = mul(parent, sub(ONE, wj))
            t[base + stride] = mul(parent, wj)
    return t


class RefProver:
    """One class for all shapes; `round` returns the EvalsInfty wire."""

    def __init__(self, kind, order, tables, w=None):
        self.kind, self.order = kind, order
        self.t = [list(t) for t in tables]
        self.r = 0
        if kind == "eqf":
            v = len(w)
            self.v, self.vl = v, v // 2
            p = list(tables[0]) + [ZERO] * ((1 << v) - len(tables[0]))
            self.t = [p, build_eq(w[: self.vl]), build_eq(w[self.vl:])]

    def degree(self):
        return {"ml": 1, "ip": 2, "eqf": 2}.get(self.kind, len(self.t))

    def _fold(self, w, which=None):
        idx = range(len(self.t)) if which is None else which
        for i in idx:
            if self.kind == "coef":
                self.t[i] = fold_msb_floor(self.t[i], w) if self.order == "msb" else fold_lsb(self.t[i], w)
            else:
                self.t[i] = fold_msb_pad(self.t[i], w) if self.order == "msb" else fold_lsb(self.t[i], w)

    def round(self, w=None):
        k = self.kind
        if k == "eqf":
            if w is not None:
                prev = self.r - 1
                self._fold(w, [0, 1] if prev < self.vl else [0, 2])
            p, el, er = self.t
            if self.r < self.vl:
                elh, m, ph = len(el) // 2, len(er), len(p) // 2
                q0, qi = ZERO, ZERO
                for a in range(elh):
                    i0, idl = ZERO, ZERO
                    for b in range(m):
                        pl, phh = p[a * m + b], p[ph + a * m + b]
                        i0 = add(i0, mul(er[b], pl))
                        idl = add(idl, mul(er[b], sub(phh, pl)))
                    q0 = add(q0, mul(el[a], i0))
                    qi = add(qi, mul(sub(el[elh + a], el[a]), idl))
            else:
                n = len(p)
                if n <= 1:
                    q0, qi = (mul(mul(el[0], er[0]), p[0]) if n == 1 else ZERO), ZERO
                else:
                    h = n // 2
                    q0, qi = ZERO, ZERO
                    for i in range(h):
                        q0 = add(q0, mul(er[i], p[i]))
                        qi = add(qi, mul(sub(er[h + i], er[i]), sub(p[h + i], p[i])))
                    q0, qi = mul(q0, el[0]), mul(qi, el[0])
            self.r += 1
            return [q0, qi]
        if w is not None:
            self._fold(w)
        self.r += 1
        if k == "ml":
            s0, _ = ml_msb_compute(self.t[0]) if self.order == "msb" else ml_lsb_compute(self.t[0])
            return [s0]
        if k == "ip":
            q = ip_msb_compute(*self.t) if self.order == "msb" else ip_lsb_compute(*self.t)
            return list(q)
        # coef: product evaluator
        n = len(self.t[0])
        half = n // 2
        d = len(self.t)
        c = [ZERO] * (d + 1)
        for j in range(half):
            il, ih = (j, j + half) if self.order == "msb" else (2 * j, 2 * j + 1)
            pc = product_coeffs([t[il] for t in self.t], [t[ih] for t in self.t])
            c = [add(x, y) for x, y in zip(c, pc)]
        if d <= 1:
            return [c[0]]
        return [c[0], c[d]] + [horner(c, lift(i)) for i in range(2, d)]

    def finalize(self, w):
        if self.kind == "eqf":
            last = self.v - 1 if self.v > 0 else 1 << 64
            self._fold(w, [0, 1] if last < self.vl else [0, 2])
        else:
            self._fold(w)

    def final_value(self):
        k = self.kind
        if k == "ml":
            return self.t[0][0] if len(self.t[0]) == 1 else ZERO
        if k == "ip":
            return mul(self.t[0][0], self.t[1][0]) if len(self.t[0]) == 1 else ZERO
        if k == "eqf":
            p, el, er = self.t
            return mul(mul(p[0], el[0]), er[0]) if len(p) == 1 else ZERO
        if len(self.t) == 1 and len(self.t[0]) == 1:
            return self.t[0][0]
        lo = [t[0] if len(t) == 1 else ZERO for t in self.t]
        c = product_coeffs(lo, [ZERO] * len(lo))
        return add(horner(c, ZERO), horner(c, ONE))


def mle_eval_msb(table, point):
    cur = list(table)
    for r in point:
        h = len(cur) // 2
        cur = [add(cur[i], mul(sub(cur[i + h], cur[i]), r)) for i in range(h)]
    return cur[0]


class RefGkr:
    """GkrProver (src/provers/gkr.rs): broadcast witness tables, every round
    folds all four tables and returns [q(0), (q(0) + q(2) - 2 q(1)) / 2]."""

    def __init__(self, add_, mult_, w):
        n = len(w)
        self.t = [list(add_), list(mult_), [w[b] for b in range(n) for _ in range(n)],
                  [w[c] for _ in range(n) for c in range(n)]]

    @staticmethod
    def term(a, m, wb, wc):
        return add(mul(a, add(wb, wc)), mul(m, mul(wb, wc)))

    def round(self, r=None):
        if r is not None:
            self.t = [fold_msb_pad(t, r) for t in self.t]
        A, M, B, C = self.t
        n = len(A)
        if n <= 1:
            return [self.term(A[0], M[0], B[0], C[0]) if n == 1 else ZERO, ZERO]
        h = np2(n) >> 1
        q = [ZERO, ZERO, ZERO]
        for i in range(h):
            lo = (A[i], M[i], B[i], C[i])
            hi = (A[i + h], M[i + h], B[i + h], C[i + h]) if i + h < n else (ZERO,) * 4
            for x in range(3):
                pt = [add(lo[j], mul(lift(x), sub(hi[j], lo[j]))) for j in range(4)]
                q[x] = add(q[x], self.term(*pt))
        inv2 = lift((P + 1) // 2)
        return [q[0], mul(sub(add(q[0], q[2]), add(q[1], q[1])), inv2)]

    def finalize(self, r):
        self.t = [fold_msb_pad(t, r) for t in self.t]

    def final_value(self):
        A, M, B, C = self.t
        return self.term(A[0], M[0], B[0], C[0]) if len(A) == 1 else ZERO



def poly_trim(c):
    c = list(c)
    while c and c[-1] == ZERO:
        c.pop()
    return c


def poly_add(p, q):
    n = max(len(p), len(q))
    return poly_trim([add(p[i] if i < len(p) else ZERO, q[i] if i < len(q) else ZERO) for i in range(n)])


def poly_sub(p, q):
    n = max(len(p), len(q))
    return poly_trim([sub(p[i] if i < len(p) else ZERO, q[i] if i < len(q) else ZERO) for i in range(n)])


def poly_mul(p, q):
    if not p or not q:
        return []
    out = [ZERO] * (len(p) + len(q) - 1)
    for i, x in enumerate(p):
        for j, y in enumerate(q):
            out[i + j] = add(out[i + j], mul(x, y))
    return poly_trim(out)


def protogalaxy_fold_naive(pairs, polys):
    """The naive fold of src/folding.rs:124-137 (tests): per level, each pair
    of neighbours becomes p0 + (a + b X) (p1 - p0), with normalised dense
    polynomials (trailing zeros dropped, zero = [])."""
    ps = [poly_trim(p) for p in polys]
    for a, b in pairs:
        ps = [poly_add(ps[2 * i], poly_mul(poly_trim([a, b]), poly_sub(ps[2 * i + 1], ps[2 * i])))
              for i in range(len(ps) // 2)]
    return ps[0]
