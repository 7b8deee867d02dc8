"""The InnerProduct start that runs rounds 0-3 in two passes over the base
tables (ip012.cuh), restated in Python big integers and checked against the
big-integer reference prover (RefProver, src/provers/inner_product.rs and
inner_product_lsb.rs, one fold + evaluate per round):

- rounds 0, 1, 2 from the 26 sums of one pass (products of the octet's
  bilinear forms on the grid {0, 1, inf}^2 and at the t2 = 1 points),
  interpolated at the challenges as the last block does;
- the octet folded with r0, r1, r2 at once as sum_s D_s prod_{i in s} r_i
  (finite differences D_s of the octet), and round 3 on those entries.
Edge values (0, 1, p - 1, 2^32) make every difference wrap.  No GPU: this
pins the algebra, the GPU tests pin the kernels."""
import random

import pytest

import bigint_ref as R

P = R.P


def quad_at(s0, s1, sinf, r):
    """q(r) of the quadratic with q(0) = s0, q(1) = s1, leading coefficient sinf."""
    c1 = R.sub(R.sub(s1, s0), sinf)
    return R.add(R.mul(R.add(R.mul(sinf, r), c1), r), s0)


def biquad_at(G, r0, r1):
    g = [quad_at(R.lift(G[v]), R.lift(G[3 + v]), R.lift(G[6 + v]), r0) for v in range(3)]
    return quad_at(g[0], g[1], g[2], r1)


def octet(X, m, O, lsb):
    """v[4 t0 + 2 t1 + t2] of octet m (base values)."""
    if lsb:
        e = X[8 * m: 8 * m + 8]
        return [e[(j >> 2) | (j & 2) | ((j & 1) << 2)] for j in range(8)]
    return [X[m + j * O] for j in range(8)]


def sums26(a, b, lsb):
    O = len(a) // 8
    S = [0] * 26
    sb = lambda x, y: (x - y) % P  # noqa: E731
    for m in range(O):
        x, y = octet(a, m, O, lsb), octet(b, m, O, lsb)
        # the t2 = 0 grid and the t2 difference grid, order (u, v) = 3u + v
        def grid(v):
            return [v[0], v[2], sb(v[2], v[0]), v[4], v[6], sb(v[6], v[4]), sb(v[4], v[0]), sb(v[6], v[2]),
                    sb(sb(v[6], v[4]), sb(v[2], v[0]))]
        gx, gy = grid(x), grid(y)
        # the t2 differences at (0,0), (0,1), (1,0), (1,1), placed where grid() reads them
        dxx = [sb(x[1], x[0]), sb(x[3], x[2]), sb(x[5], x[4]), sb(x[7], x[6])]
        dyy = [sb(y[1], y[0]), sb(y[3], y[2]), sb(y[5], y[4]), sb(y[7], y[6])]
        dx = grid([dxx[0], 0, dxx[1], 0, dxx[2], 0, dxx[3], 0])
        dy = grid([dyy[0], 0, dyy[1], 0, dyy[2], 0, dyy[3], 0])
        for g in range(9):
            S[g] += gx[g] * gy[g]
            S[14 + g] += dx[g] * dy[g]
        S[9] += x[1] * y[1]
        S[10] += x[5] * y[5]
        S[11] += sb(x[5], x[1]) * sb(y[5], y[1])
        S[12] += x[3] * y[3]
        S[13] += sb(x[7], x[3]) * sb(y[7], y[3])
        e0, f0 = sb(x[3], x[1]), sb(y[3], y[1])
        e1, f1 = sb(x[7], x[5]), sb(y[7], y[5])
        S[23] += e0 * f0
        S[24] += e1 * f1
        S[25] += sb(e1, e0) * sb(f1, f0)
    return [s % P for s in S]


def wires_012(S, r0, r1):
    ad = lambda *v: sum(v) % P  # noqa: E731
    w0 = (R.lift(ad(S[0], S[1], S[9], S[12])), R.lift(ad(S[6], S[7], S[11], S[13])))
    w1 = (quad_at(R.lift(ad(S[0], S[9])), R.lift(ad(S[3], S[10])), R.lift(ad(S[6], S[11])), r0),
          quad_at(R.lift(ad(S[2], S[23])), R.lift(ad(S[5], S[24])), R.lift(ad(S[8], S[25])), r0))
    w2 = (biquad_at(S[0:9], r0, r1), biquad_at(S[14:23], r0, r1))
    return [w0, w1, w2]


def fold3(v, r0, r1, r2):
    d = list(v)
    for j in range(4, 8):
        d[j] = (d[j] - d[j - 4]) % P
    for j in range(8):
        if j & 2:
            d[j] = (d[j] - d[j - 2]) % P
    for j in range(8):
        if j & 1:
            d[j] = (d[j] - d[j - 1]) % P
    K = {4: r0, 2: r1, 1: r2, 6: R.mul(r0, r1), 5: R.mul(r0, r2), 3: R.mul(r1, r2)}
    K[7] = R.mul(K[6], r2)
    out = R.lift(d[0])
    for j in range(1, 8):
        out = R.add(out, R.mul(R.lift(d[j]), K[j]))
    return out


EDGE = [0, 1, P - 1, 1 << 32, P - 2, (1 << 32) - 1]


@pytest.mark.parametrize("n", [3, 4, 5, 6])
@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("edge", [False, True])
def test_rounds_0_3_forms(n, order, edge):
    rng = random.Random(1000 * n + (order == "lsb") * 7 + edge)
    L = 1 << n
    pick = (lambda: rng.choice(EDGE)) if edge else (lambda: rng.randrange(P))
    a = [pick() for _ in range(L)]
    b = [pick() for _ in range(L)]
    rs = [(rng.randrange(P), rng.randrange(P), rng.randrange(P)) for _ in range(3)]
    ref = R.RefProver("ip", order, [[R.lift(x) for x in a], [R.lift(x) for x in b]])
    want = [ref.round(None), ref.round(rs[0]), ref.round(rs[1])]
    lsb = order == "lsb"
    got = wires_012(sums26(a, b, lsb), rs[0], rs[1])
    for rd in range(3):
        assert tuple(got[rd][0]) == tuple(want[rd][0]), ("q0", rd)
        assert tuple(got[rd][1]) == tuple(want[rd][1]), ("qinf", rd)
    # the triple fold gives the reference's tables after rounds 0-3's folds
    # and round 3's wire
    want3 = ref.round(rs[2])
    O = L // 8
    A3 = [fold3(octet(a, m, O, lsb), *rs) for m in range(O)]
    B3 = [fold3(octet(b, m, O, lsb), *rs) for m in range(O)]
    assert A3 == [tuple(x) for x in ref.t[0]]
    assert B3 == [tuple(x) for x in ref.t[1]]
    q3 = R.ip_lsb_compute(A3, B3) if lsb else R.ip_msb_compute(A3, B3)
    assert tuple(q3[0]) == tuple(want3[0]) and tuple(q3[1]) == tuple(want3[1])
