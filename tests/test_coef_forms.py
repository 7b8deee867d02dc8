"""The Coefficient (degree-3 product evaluator) start that runs rounds 0-2
in two passes over the input tables (coef01.cuh), restated in Python big
integers and checked against the big-integer reference prover (RefProver
"coef", src/provers/coefficient.rs and coefficient_lsb.rs, one fold +
evaluate per round):

- rounds 0 and 1 from 15 sums of one pass: per quadruple, every table's
  bilinear form F(y, x) (y the round-0 variable, x round 1's) at the grid
  points (y, x) in {0, 1, 2, inf} x {0, 2, inf} and at (u, 1) for
  u in {0, 2, inf}, multiplied across the three tables and summed; round 0
  from the x in {0, 1} columns, round 1 by interpolating each x column (a
  cubic in y) at r0;
- the quadruple folded with r0 and r1 at once (t00 + r0 d10 + r1 d01 +
  r0 r1 d11), and round 2 on those entries.
Edge values (0, 1, p - 1) make the differences wrap.  No GPU: this pins
the algebra, the GPU tests pin the kernels."""
import random

import pytest

import bigint_ref as R

P = R.P
INV2 = (P + 1) // 2
INF = "inf"
Y_PTS = (0, 1, 2, INF)
X_PTS = (0, 2, INF)


def forms(t):
    """(t00, d10, d01, d11) of a quadruple t[u][v] (Fp3 tuples)."""
    t00, t01, t10, t11 = t[0][0], t[0][1], t[1][0], t[1][1]
    d10, d01 = R.sub(t10, t00), R.sub(t01, t00)
    d11 = R.add(R.sub(R.sub(t11, t10), t01), t00)
    return t00, d10, d01, d11


def F(f, y, x):
    """The bilinear form at (y, x); inf takes the leading coefficient."""
    t00, d10, d01, d11 = f
    sc = lambda v, k: R.mul(v, R.lift(k))  # noqa: E731
    if y == INF and x == INF:
        return d11
    if y == INF:
        return R.add(d10, sc(d11, x))
    if x == INF:
        return R.add(d01, sc(d11, y))
    return R.add(R.add(t00, sc(d10, y)), R.add(sc(d01, x), sc(d11, x * y)))


def points():
    """The 15 product points: the 4 x 3 grid, then (u, 1) for u in {0, 2, inf}."""
    return [(y, x) for x in X_PTS for y in Y_PTS] + [(u, 1) for u in (0, 2, INF)]


def quads(T, order):
    """Per quadruple index k: t[u][v] with u the round-0 bit, v round 1's."""
    L = len(T)
    Q = L // 4
    out = []
    for k in range(Q):
        if order == "msb":
            out.append([[T[k], T[k + Q]], [T[k + 2 * Q], T[k + 3 * Q]]])
        else:
            out.append([[T[4 * k], T[4 * k + 2]], [T[4 * k + 1], T[4 * k + 3]]])
    return out


def sums15(tables, order):
    qs = [quads(T, order) for T in tables]
    S = [R.ZERO] * 15
    for k in range(len(qs[0])):
        fs = [forms(q[k]) for q in qs]
        for i, (y, x) in enumerate(points()):
            p = R.ONE
            for f in fs:
                p = R.mul(p, F(f, y, x))
            S[i] = R.add(S[i], p)
    return S


def cubic_at(g0, g1, g2, ginf, r):
    """G(r) of the cubic with G(0), G(1), G(2) and leading coefficient ginf:
    ginf r (r-1)(r-2) + g0 (r-1)(r-2)/2 - g1 r (r-2) + g2 r (r-1)/2."""
    one, two = R.ONE, R.lift(2)
    r1, r2 = R.sub(r, one), R.sub(r, two)
    h = R.lift(INV2)
    t = R.mul(R.mul(ginf, r), R.mul(r1, r2))
    t = R.add(t, R.mul(R.mul(g0, h), R.mul(r1, r2)))
    t = R.sub(t, R.mul(g1, R.mul(r, r2)))
    t = R.add(t, R.mul(R.mul(g2, h), R.mul(r, r1)))
    return t


def round01(S, r0):
    """Round 0's wire, and round 1's at the challenge r0: [h(0), h(inf), h(2)]."""
    idx = {pt: i for i, pt in enumerate(points())}
    h0 = {u: R.add(S[idx[(u, 0)]], S[idx[(u, 1)]]) for u in (0, 2, INF)}
    w0 = [h0[0], h0[INF], h0[2]]
    h1 = {x: cubic_at(S[idx[(0, x)]], S[idx[(1, x)]], S[idx[(2, x)]], S[idx[(INF, x)]], r0) for x in X_PTS}
    w1 = [h1[0], h1[INF], h1[2]]
    return w0, w1


def fold2(T, order, r0, r1):
    """Every table folded with r0 then r1 at once: t00 + r0 d10 + r1 d01 + r0 r1 d11."""
    out = []
    for q in quads(T, order):
        t00, d10, d01, d11 = forms(q)
        out.append(R.add(R.add(t00, R.mul(r0, d10)), R.add(R.mul(r1, d01), R.mul(R.mul(r0, r1), d11))))
    return out


def rnd_tables(rng, n, ext0, edges):
    def el(ext):
        if edges and rng.random() < 0.3:
            v = rng.choice([0, 1, P - 1])
        else:
            v = rng.randrange(P)
        return (v, rng.randrange(P), rng.randrange(P)) if ext else (v, 0, 0)
    return [[el(ext0 if t == 0 else False) for _ in range(n)] for t in range(3)]


@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("n", [4, 8, 16, 32])
@pytest.mark.parametrize("ext0", [True, False])
@pytest.mark.parametrize("edges", [False, True])
def test_two_pass_start_matches_reference(order, n, ext0, edges):
    rng = random.Random(n * 10 + (order == "lsb") + 2 * ext0 + 4 * edges)
    tables = rnd_tables(rng, n, ext0, edges)
    ref = R.RefProver("coef", order, tables)
    r0 = (rng.randrange(P), rng.randrange(P), rng.randrange(P))
    r1 = (rng.randrange(P), rng.randrange(P), rng.randrange(P))
    w0_ref = ref.round()
    w1_ref = ref.round(r0)
    w2_ref = ref.round(r1)
    S = sums15(tables, order)
    w0, w1 = round01(S, r0)
    assert w0 == w0_ref
    assert w1 == w1_ref
    T2 = [fold2(T, order, r0, r1) for T in tables]
    assert T2 == ref.t
    # round 2 on the double-folded tables is the reference's round 2
    chk = R.RefProver("coef", order, T2)
    assert chk.round() == w2_ref


def test_cubic_interpolation():
    rng = random.Random(3)
    for _ in range(50):
        c = [(rng.randrange(P), rng.randrange(P), rng.randrange(P)) for _ in range(4)]
        r = (rng.randrange(P), rng.randrange(P), rng.randrange(P))
        g = [R.horner(c, R.lift(v)) for v in (0, 1, 2)]
        assert cubic_at(g[0], g[1], g[2], c[3], r) == R.horner(c, r)
