"""The GkrProver forms the device kernels evaluate, restated in Python big
integers and checked against the big-integer reference (RefGkr, the
broadcast tables and three evaluation points of src/provers/gkr.rs:105-190):

- every round's wire [q(0), (q(0) + q(2) - 2 q(1)) / 2] as q(0) and the x^2
  coefficient c2 = sum d_w (d_add + d_mult s) on the compact witness tables;
- rounds 0 and 1 from the eight base sums of one pass over quadruples, per
  quadruple and per run of quadruples sharing one W_b entry;
- a b-variable round from per-run sums finished with the run's W_b entries.
No GPU: this pins the algebra, the GPU tests pin the kernels."""
import random

import pytest

import bigint_ref as R

P = R.P
INV2 = (P + 1) // 2


def rand_gkr(k, seed, ext=False):
    rng = random.Random(seed)
    n = 1 << k
    el = (lambda: (rng.randrange(P), rng.randrange(P), rng.randrange(P))) if ext else (lambda: R.lift(rng.randrange(P)))
    return rng, [el() for _ in range(n * n)], [el() for _ in range(n * n)], [el() for _ in range(n)]


def chal(rng):
    return (rng.randrange(P), rng.randrange(P), rng.randrange(P))


@pytest.mark.parametrize("k", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("ext", [False, True])
def test_q0_c2_every_round(k, ext):
    """Compact W_b / W_c (W_b[i >> kc], W_c[i & (2^kc - 1)]) and the two
    accumulated values give the reference's wire in every round, including
    rounds past 2k (tables of one entry: c2 = 0)."""
    rng, A, M, w = rand_gkr(k, 10 + k + ext, ext)
    ref = R.RefGkr(A, M, w)
    WB, WC = list(w), list(w)
    r = None
    for rd in range(2 * k + 2):
        want = ref.round(r)
        if r is not None:
            if rd - 1 < k:
                WB = R.fold_msb_pad(WB, r)
            else:
                WC = R.fold_msb_pad(WC, r)
            A, M = R.fold_msb_pad(A, r), R.fold_msb_pad(M, r)
        Ln = len(A)
        lg = Ln.bit_length() - 1
        kc = min(k, lg)
        cm = (1 << kc) - 1
        if Ln == 1:
            got = [R.RefGkr.term(A[0], M[0], WB[0], WC[0]), R.ZERO]
        else:
            H = Ln >> 1
            bvar = kc < lg
            q0, c2 = R.ZERO, R.ZERO
            for i in range(H):
                wbl, wcl = WB[i >> kc], WC[i & cm]
                q0 = R.add(q0, R.RefGkr.term(A[i], M[i], wbl, wcl))
                da, dm = R.sub(A[i + H], A[i]), R.sub(M[i + H], M[i])
                if bvar:
                    assert WC[(i + H) & cm] == wcl
                    dw, s = R.sub(WB[(i + H) >> kc], wbl), wcl
                else:
                    assert WB[(i + H) >> kc] == wbl
                    dw, s = R.sub(WC[(i + H) & cm], wcl), wbl
                c2 = R.add(c2, R.mul(dw, R.add(da, R.mul(dm, s))))
            got = [q0, c2]
        assert got == want, (k, rd)
        r = chal(rng)


def first_two_wires(s, r0):
    """finalize of the eight sums (T0, T1, T2, U0, U1, U2, V0, V2)."""
    L = R.lift
    w0 = [L((s[0] + s[6]) % P), L((s[2] + s[7]) % P)]
    q0 = R.add(R.mul(R.add(R.mul(L(s[2]), r0), L(s[1])), r0), L(s[0]))
    qi = R.add(R.mul(R.add(R.mul(L(s[5]), r0), L(s[4])), r0), L(s[3]))
    return w0, [q0, qi]


def base_gkr(k, seed):
    rng = random.Random(seed)
    n = 1 << k
    return (rng, [rng.randrange(P) for _ in range(n * n)], [rng.randrange(P) for _ in range(n * n)],
            [rng.randrange(P) for _ in range(n)])


@pytest.mark.parametrize("k", [2, 3, 4])
@pytest.mark.parametrize("run", [0, 4, 16])
def test_rounds_0_1_from_eight_sums(k, run):
    """Per quadruple j < N/4 (x_s = x[j + s N/4], w_s = W[(j >> k) + s n/4],
    c = W[j mod n]) or per run of `run` quadruples sharing one b."""
    n = 1 << k
    if run > n:
        pytest.skip("a run stays inside one b")
    rng, add_, mult_, w = base_gkr(k, 100 * k + run)
    ref = R.RefGkr([R.lift(x) for x in add_], [R.lift(x) for x in mult_], [R.lift(x) for x in w])
    wire0 = ref.round()
    r0 = chal(rng)
    wire1 = ref.round(r0)
    Q, nq = n * n // 4, n // 4
    s = [0] * 8
    if run == 0:
        for j in range(Q):
            a0, a1, a2, a3 = (add_[j + t * Q] for t in range(4))
            m0, m1, m2, m3 = (mult_[j + t * Q] for t in range(4))
            b = j >> k
            w0, w1, w2, w3 = (w[b + t * nq] for t in range(4))
            c = w[j & (n - 1)]
            da0, da1, dm0, dm1 = a2 - a0, a3 - a1, m2 - m0, m3 - m1
            dw0, dw1 = w2 - w0, w3 - w1
            s[0] += a0 * (w0 + c) + c * m0 * w0
            s[6] += a1 * (w1 + c) + c * m1 * w1
            s[2] += dw0 * (da0 + c * dm0)
            s[7] += dw1 * (da1 + c * dm1)
            s[1] += c * (m0 * dw0 + dm0 * w0) + a0 * dw0 + da0 * (w0 + c)
            e, f = w1 - w0, dw1 - dw0
            g, h = (a1 - a0) + c * (m1 - m0), (da1 - da0) + c * (dm1 - dm0)
            s[3] += e * g
            s[4] += f * g + e * h
            s[5] += f * h
    else:
        for u in range(Q // run):
            i0 = u * run
            b = i0 >> k
            X, C = [0] * 4, [0] * 3
            for j in range(i0, i0 + run):
                assert j >> k == b
                c = w[j & (n - 1)]
                for t in range(4):
                    X[t] += add_[j + t * Q] + c * mult_[j + t * Q]
                for t in range(3):
                    C[t] += c * add_[j + t * Q]
            w0, w1, w2, w3 = (w[b + t * nq] for t in range(4))
            dw0, dw1, e = w2 - w0, w3 - w1, w1 - w0
            f = dw1 - dw0
            d20, d31 = X[2] - X[0], X[3] - X[1]
            g, h = X[1] - X[0], d31 - d20
            s[0] += w0 * X[0] + C[0]
            s[6] += w1 * X[1] + C[1]
            s[2] += dw0 * d20
            s[7] += dw1 * d31
            s[1] += dw0 * X[0] + w0 * d20 + C[2] - C[0]
            s[3] += e * g
            s[4] += f * g + e * h
            s[5] += f * h
    s = [x % P for x in s]
    assert first_two_wires(s, r0) == (wire0, wire1)


@pytest.mark.parametrize("k,run", [(3, 8), (4, 4), (4, 16), (5, 32)])
def test_b_round_by_runs(k, run):
    """A b-variable round from the run sums sum (add + mult s), sum add s and
    sum (d_add + d_mult s), finished with wl and wh of the run."""
    rng, A, M, w = rand_gkr(k, 7 * k + run, ext=True)
    w = [R.lift(x[0]) for x in w]
    ref = R.RefGkr(A, M, w)
    n = 1 << k
    WB, WC = list(w), list(w)
    r = None
    checked = 0
    for rd in range(k):
        want = ref.round(r)
        if r is not None:
            WB, A, M = R.fold_msb_pad(WB, r), R.fold_msb_pad(A, r), R.fold_msb_pad(M, r)
        H = len(A) >> 1
        if run <= n and H % run == 0:
            q0, c2 = R.ZERO, R.ZERO
            for u in range(H // run):
                i0 = u * run
                xa, ya, zd = R.ZERO, R.ZERO, R.ZERO
                for i in range(i0, i0 + run):
                    s = WC[i & (n - 1)]
                    xa = R.add(xa, R.add(A[i], R.mul(M[i], s)))
                    ya = R.add(ya, R.mul(A[i], s))
                    zd = R.add(zd, R.add(R.sub(A[i + H], A[i]), R.mul(R.sub(M[i + H], M[i]), s)))
                wl, wh = WB[i0 >> k], WB[(i0 + H) >> k]
                q0 = R.add(q0, R.add(R.mul(xa, wl), ya))
                c2 = R.add(c2, R.mul(zd, R.sub(wh, wl)))
            assert [q0, c2] == want, (k, rd)
            checked += 1
        r = chal(rng)
    assert checked
