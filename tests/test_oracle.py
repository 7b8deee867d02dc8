"""CPU tests: pin the oracle.

The reference crate holds no golden vectors (its tests are property tests), so
the oracle is pinned three ways:
  * field arithmetic against Python big integers and the Montgomery
    known-answer constants of the reference (src/tests/fields.rs:62-63);
  * the Keccak permutation against hashlib's SHA3-256;
  * every prover, round by round, against the independent big-integer
    restatement in ``bigint_ref.py``; and the reference's own property tests
    (fused == unfused, MLE at the challenges, split == full, verifier
    acceptance/rejection, EqFactored == InnerProduct(eq table),
    Coefficient(deg 1) == Multilinear, LSB/MSB prove the same sum).
"""
import hashlib
import random

import numpy as np
import pytest

import bigint_ref as R
from oracle import oracle as O

P = R.P


def rnd_f(rng, ext=True):
    return (rng.randrange(P), rng.randrange(P) if ext else 0, rng.randrange(P) if ext else 0)


def to_np(vals):
    return np.array([list(v) for v in vals], dtype=np.uint64).reshape(-1, 3)


def tup(a):
    return tuple(int(x) for x in np.asarray(a).reshape(3))


# ---------------------------------------------------------------- field ------
def test_constants_and_montgomery_kats():
    assert O.W == R.W == 0xFFFFFFF800000001
    lib = O.lib()
    # mont(1) = eps, mont(-1) = p - eps (reference src/tests/fields.rs:62-63)
    assert lib.or_fp_to_mont(1) == 0xFFFFFFFF
    assert lib.or_fp_to_mont(P - 1) == 0xFFFFFFFE00000002
    assert lib.or_fp_from_mont(7) == R.W
    # W is a non-cube, so X^3 - W is irreducible and Fp3 is a field
    assert pow(R.W, (P - 1) // 3, P) != 1
    for x in [0, 1, 2, P - 1, P - 2, 0xFFFFFFFF, 1 << 32, 1 << 63]:
        assert lib.or_fp_from_mont(lib.or_fp_to_mont(x)) == x
        assert lib.or_fp_to_mont(x) == x * (1 << 64) % P


def test_fp_ops_match_bigint():
    rng = random.Random(1)
    lib = O.lib()
    edge = [0, 1, 2, P - 1, P - 2, (1 << 32) - 1, 1 << 32, (1 << 32) + 1, (1 << 63), P - (1 << 32)]
    vals = edge + [rng.randrange(P) for _ in range(3000)]
    for i in range(len(vals)):
        a, b = vals[i], vals[(i * 7 + 3) % len(vals)]
        assert lib.or_fp_add(a, b) == (a + b) % P
        assert lib.or_fp_sub(a, b) == (a - b) % P
        assert lib.or_fp_mul(a, b) == a * b % P
    for a in edge[1:] + vals[-50:]:
        if a:
            assert lib.or_fp_inv(a) == pow(a, -1, P)


def test_fp3_mul_matches_bigint():
    rng = random.Random(2)
    for _ in range(2000):
        a, b = rnd_f(rng), rnd_f(rng)
        assert tup(O.f3_mul(a, b)) == R.mul(a, b)
    # X * X^2 = W
    assert tup(O.f3_mul((0, 1, 0), (0, 0, 1))) == (R.W, 0, 0)


# --------------------------------------------------------------- keccak ------
@pytest.mark.parametrize("n", [0, 1, 3, 135, 136, 137, 200, 271, 272, 273, 1000])
def test_keccak_sponge_matches_sha3(n):
    msg = bytes((i * 31 + 7) & 0xFF for i in range(n))
    assert O.sha3_256(msg) == hashlib.sha3_256(msg).digest()


def test_transcript_deterministic_and_label_separated():
    t1 = O.Transcript(3, label=b"effsc-gpu/ip/v1")
    t2 = O.Transcript(3, label=b"effsc-gpu/ip/v1")
    t3 = O.Transcript(3, label=b"effsc-gpu/ip/v2")
    for t in (t1, t2, t3):
        t.send((1, 2, 3))
    c1, c2, c3 = t1.challenge(), t2.challenge(), t3.challenge()
    assert (c1 == c2).all() and not (c1 == c3).all()
    assert all(int(x) < P for x in c1)


# ----------------------------------------------------------- generator ------
def test_generator_uniform_canonical():
    t = O.gen_table(12345, 1 << 16)
    assert (t < np.uint64(P)).all()
    assert len(np.unique(t)) == t.size
    # element i is SplitMix64 output i of the seeded stream
    s = 12345
    x = s
    for i in range(4):
        x = (x + 0x9E3779B97F4A7C15) & (2**64 - 1)
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2**64 - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2**64 - 1)
        z ^= z >> 31
        assert int(t[i]) == z


# ------------------------------------------------------ provers vs bigint ---
def make_tables(rng, k, n, ext):
    return [[rnd_f(rng, ext) for _ in range(n)] for _ in range(k)]


CASES = [
    ("ml", "msb", 1), ("ml", "lsb", 1), ("ip", "msb", 2), ("ip", "lsb", 2),
    ("coef", "msb", 3), ("coef", "lsb", 3), ("coef", "msb", 1), ("coef", "lsb", 2),
]
KIND = {"ml": O.ML, "ip": O.IP, "coef": O.COEF}
ORD = {"msb": O.MSB, "lsb": O.LSB}


@pytest.mark.parametrize("kind,order,k", CASES)
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 13, 16, 33, 64])
@pytest.mark.parametrize("ext", [False, True])
def test_prover_rounds_match_bigint(kind, order, k, n, ext):
    if kind == "ip" and order == "lsb" and n % 2 and n > 1:
        pytest.skip("reference compute_lsb indexes past the end for odd lengths")
    rng = random.Random(hash((kind, order, k, n, ext)) & 0xFFFF)
    tabs = make_tables(rng, k, n, ext)
    ref = R.RefProver(kind, order, tabs)
    orc = O.Prover(KIND[kind], ORD[order], 3, [to_np(t) for t in tabs])
    rounds = max(1, (n - 1).bit_length()) + 1  # one extra round beyond log2
    w = None
    for _ in range(rounds):
        a = ref.round(w)
        b = orc.round(w)
        assert [tuple(int(x) for x in row) for row in b] == a
        w = rnd_f(rng, True)
    ref.finalize(w)
    orc.finalize(w)
    assert tup(orc.final_value()) == ref.final_value()


@pytest.mark.parametrize("v", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("plen_frac", [1.0, 0.5])
def test_eq_factored_rounds_match_bigint(v, plen_frac):
    rng = random.Random(100 + v)
    w = [rnd_f(rng) for _ in range(v)]
    plen = max(1, int((1 << v) * plen_frac))
    p = [rnd_f(rng, False) for _ in range(plen)]
    ref = R.RefProver("eqf", "msb", [p], w=w)
    orc = O.Prover.eq_factored(3, to_np(w) if v else np.zeros((0, 3), np.uint64), to_np(p))
    ch = None
    for _ in range(v):
        assert [tuple(int(x) for x in row) for row in orc.round(ch)] == ref.round(ch)
        ch = rnd_f(rng)
    if v:
        ref.finalize(ch)
        orc.finalize(ch)
    assert tup(orc.final_value()) == ref.final_value()


def test_eq_table_matches_bigint_and_sums_to_one():
    rng = random.Random(5)
    w = [rnd_f(rng) for _ in range(5)]
    t = O.build_eq_table(to_np(w))
    assert [tuple(int(x) for x in r) for r in t] == R.build_eq(w)
    s = R.ZERO
    for r in t:
        s = R.add(s, tuple(int(x) for x in r))
    assert s == R.ONE


# ------------------------------------------------- reference property tests --
def run(prover, n_rounds, label=b"t", deg=3, hook=b"", seed=None, legacy=False):
    t = O.Transcript(deg, seed=seed) if seed is not None else O.Transcript(deg, label=label)
    return O.sumcheck(prover, n_rounds, t, hook=hook, legacy=legacy)


def claimed_sum_ip(a, b):
    s = R.ZERO
    for x, y in zip(a, b):
        s = R.add(s, R.mul(x, y))
    return s


@pytest.mark.parametrize("deg", [1, 3])
@pytest.mark.parametrize("order", [O.MSB, O.LSB])
def test_ip_full_roundtrip_verifies_and_mle(deg, order):
    rng = random.Random(7)
    v = 8
    a = [rnd_f(rng, False) for _ in range(1 << v)]
    b = [rnd_f(rng, False) for _ in range(1 << v)]
    pr = O.Prover(O.IP, order, deg, [to_np(a), to_np(b)])
    rp, ch, fv = run(pr, v, deg=deg, label=b"effsc-gpu/ip/v1")
    cl, fc = O.verify(claimed_sum_ip(a, b), 2, v, O.Transcript(deg, label=b"effsc-gpu/ip/v1"), rp)
    assert (cl == ch).all() and (fc == fv).all()
    if deg == 1:
        assert (ch[:, 1:] == 0).all()
    if order == O.MSB:
        fa = O.mle_eval_msb(to_np(a), ch)
        fb = O.mle_eval_msb(to_np(b), ch)
        assert tup(fv) == R.mul(tup(fa), tup(fb))
    # corrupt round 3's q(0): verifier returns a claim that no longer matches
    rp2 = rp.copy()
    rp2[3, 0, 0] = (int(rp2[3, 0, 0]) + 1) % P
    _, fc2 = O.verify(claimed_sum_ip(a, b), 2, v, O.Transcript(deg, label=b"effsc-gpu/ip/v1"), rp2)
    assert not (fc2 == fv).all()


@pytest.mark.parametrize("order", [O.MSB, O.LSB])
def test_ml_roundtrip_mle_and_verify(order):
    rng = random.Random(8)
    v = 7
    e = [rnd_f(rng, False) for _ in range(1 << v)]
    pr = O.Prover(O.ML, order, 1, [to_np(e)])
    rp, ch, fv = run(pr, v, deg=1)
    s = R.ZERO
    for x in e:
        s = R.add(s, x)
    _, fc = O.verify(s, 1, v, O.Transcript(1, label=b"t"), rp)
    assert (fc == fv).all()
    if order == O.MSB:
        assert (O.mle_eval_msb(to_np(e), ch) == fv).all()
    assert pr.table(0).shape[0] == 1 and (pr.table(0)[0] == fv).all()


@pytest.mark.parametrize("kind", [O.ML, O.IP])
def test_partial_then_continue_equals_full(kind):
    rng = random.Random(9)
    v, split = 8, 3
    tabs = [to_np([rnd_f(rng, False) for _ in range(1 << v)]) for _ in range(1 if kind == O.ML else 2)]
    full = O.Prover(kind, O.MSB, 3, tabs)
    t = O.Transcript(3, label=b"split")
    rp_f, ch_f, fv_f = O.sumcheck(full, v, t)
    part = O.Prover(kind, O.MSB, 3, tabs)
    t2 = O.Transcript(3, label=b"split")
    rp1, ch1, _ = O.sumcheck(part, split, t2)
    rp2, ch2, fv2 = O.sumcheck(part, v - split, t2)
    assert (np.concatenate([rp1, rp2]) == rp_f).all()
    assert (np.concatenate([ch1, ch2]) == ch_f).all()
    assert (fv2 == fv_f).all()


def test_zero_rounds_is_identity():
    rng = random.Random(10)
    a = to_np([rnd_f(rng, False) for _ in range(8)])
    b = to_np([rnd_f(rng, False) for _ in range(8)])
    pr = O.Prover(O.IP, O.MSB, 3, [a, b])
    rp, ch, fv = run(pr, 0)
    assert rp.shape[0] == 0 and ch.shape[0] == 0
    assert (pr.table(0) == a).all() and (pr.table(1) == b).all()
    assert (fv == 0).all()


def test_ip_round0_difference_form():
    rng = random.Random(11)
    n = 16
    a = [rnd_f(rng, False) for _ in range(n)]
    b = [rnd_f(rng, False) for _ in range(n)]
    pr = O.Prover(O.IP, O.MSB, 1, [to_np(a), to_np(b)])
    out = pr.round(None)
    h = n // 2
    c0, c2 = R.ZERO, R.ZERO
    for i in range(h):
        c0 = R.add(c0, R.mul(a[i], b[i]))
        c2 = R.add(c2, R.mul(R.sub(a[i + h], a[i]), R.sub(b[i + h], b[i])))
    assert tup(out[0]) == c0 and tup(out[1]) == c2


@pytest.mark.parametrize("v", [1, 2, 3, 4, 5, 6, 7, 8])
def test_eq_factored_equals_inner_product_on_eq_table(v):
    rng = random.Random(0xE05 ^ v)
    w = to_np([rnd_f(rng) for _ in range(v)])
    p = to_np([rnd_f(rng, False) for _ in range(1 << v)])
    eqp = O.Prover.eq_factored(3, w, p)
    r1 = run(eqp, v, label=b"eqf")
    ipp = O.Prover(O.IP, O.MSB, 3, [p, O.build_eq_table(w)])
    r2 = run(ipp, v, label=b"eqf")
    for x, y in zip(r1, r2):
        assert (x == y).all()


@pytest.mark.parametrize("order", [O.MSB, O.LSB])
def test_coefficient_degree1_equals_multilinear(order):
    rng = random.Random(12)
    e = to_np([rnd_f(rng, False) for _ in range(16)])
    r1 = run(O.Prover(O.ML, order, 1, [e]), 4, deg=1, seed=99)
    r2 = run(O.Prover(O.COEF, order, 1, [e]), 4, deg=1, seed=99)
    for x, y in zip(r1, r2):
        assert (x == y).all()


@pytest.mark.parametrize("order", [O.MSB, O.LSB])
def test_coefficient_degree3_verifies(order):
    rng = random.Random(13)
    v = 6
    tabs = [[rnd_f(rng, False) for _ in range(1 << v)] for _ in range(3)]
    s = R.ZERO
    for x, y, z in zip(*tabs):
        s = R.add(s, R.mul(R.mul(x, y), z))
    pr = O.Prover(O.COEF, order, 3, [to_np(t) for t in tabs])
    hook = bytes(range(32))
    rp, ch, fv = run(pr, v, label=b"c3", hook=hook)
    assert rp.shape == (v, 3, 3)
    _, fc = O.verify(s, 3, v, O.Transcript(3, label=b"c3"), rp, hook=hook)
    assert (fc == fv).all()
    rp2 = rp.copy()
    rp2[2, 2, 1] = (int(rp2[2, 2, 1]) + 5) % P
    _, fc2 = O.verify(s, 3, v, O.Transcript(3, label=b"c3"), rp2, hook=hook)
    assert not (fc2 == fv).all()


def test_eq_factored_verifies_and_final_factors():
    rng = random.Random(14)
    v = 7
    w = [rnd_f(rng) for _ in range(v)]
    p = [rnd_f(rng, False) for _ in range(1 << v)]
    eq = R.build_eq(w)
    s = R.ZERO
    for x, y in zip(eq, p):
        s = R.add(s, R.mul(x, y))
    pr = O.Prover.eq_factored(3, to_np(w), to_np(p))
    rp, ch, fv = run(pr, v, label=b"eqf")
    _, fc = O.verify(s, 2, v, O.Transcript(3, label=b"eqf"), rp)
    assert (fc == fv).all()
    # eq(w, r) = prod (r_j w_j + (1 - r_j)(1 - w_j))
    e = R.ONE
    for j in range(v):
        r = tup(ch[j])
        e = R.mul(e, R.add(R.mul(r, w[j]), R.mul(R.sub(R.ONE, r), R.sub(R.ONE, w[j]))))
    assert tup(fv) == R.mul(e, R.mle_eval_msb(p, [tup(c) for c in ch]))


@pytest.mark.parametrize("n", [3, 5, 13, 33, 100])
def test_non_pow2_ip_msb_matches_unfused_and_verifies(n):
    rng = random.Random(n)
    a = [rnd_f(rng, False) for _ in range(n)]
    b = [rnd_f(rng, False) for _ in range(n)]
    v = (n - 1).bit_length()
    pr = O.Prover(O.IP, O.MSB, 3, [to_np(a), to_np(b)])
    rp, ch, fv = run(pr, v, label=b"np2")
    ref = R.RefProver("ip", "msb", [a, b])
    w = None
    for r in range(v):
        assert [tuple(int(x) for x in row) for row in rp[r]] == ref.round(w)
        w = tup(ch[r])
    ref.finalize(w)
    assert tup(fv) == ref.final_value()
    _, fc = O.verify(claimed_sum_ip(a, b), 2, v, O.Transcript(3, label=b"np2"), rp)
    assert (fc == fv).all()


def test_ip_lsb_rejects_odd_round0():
    rng = random.Random(15)
    a = to_np([rnd_f(rng, False) for _ in range(5)])
    pr = O.Prover(O.IP, O.LSB, 1, [a, a])
    with pytest.raises(ValueError):
        pr.round(None)


def test_legacy_ml_sends_s0_s1():
    rng = random.Random(16)
    e = [rnd_f(rng, False) for _ in range(16)]
    rp, ch, fv = run(O.Prover(O.ML, O.MSB, 1, [to_np(e)]), 4, deg=1, legacy=True)
    s0, s1 = R.ml_msb_compute(e)
    assert tup(rp[0, 0]) == s0 and tup(rp[0, 1]) == s1
    for r in range(4):
        assert R.add(tup(rp[r, 0]), tup(rp[r, 1])) == (
            R.add(s0, s1) if r == 0 else
            R.add(tup(rp[r - 1, 0]), R.mul(tup(ch[r - 1]), R.sub(tup(rp[r - 1, 1]), tup(rp[r - 1, 0])))))


# ------------------------------------------------------------- GKR -----------
def gkr_inputs(rng, k, ext=False, zero_mult=False, zero_all=False):
    n = 1 << k
    add_ = [R.ZERO if zero_all else rnd_f(rng, ext) for _ in range(n * n)]
    mult_ = [R.ZERO if (zero_mult or zero_all) else rnd_f(rng, ext) for _ in range(n * n)]
    w = [rnd_f(rng, ext) for _ in range(n)]
    return add_, mult_, w


@pytest.mark.parametrize("k", [0, 1, 2, 3])
@pytest.mark.parametrize("ext", [False, True])
@pytest.mark.parametrize("extra", [0, -1, 1])
def test_gkr_rounds_match_bigint(k, ext, extra):
    """src/provers/gkr.rs round by round (full, partial and one extra round)."""
    rng = random.Random(50 + 10 * k + ext + 3 * extra)
    add_, mult_, w = gkr_inputs(rng, k, ext)
    ref = R.RefGkr(add_, mult_, w)
    pr = O.Prover.gkr(3, to_np(add_), to_np(mult_), to_np(w))
    rounds = max(0, 2 * k + extra)
    r = None
    for j in range(rounds):
        want = ref.round(r)
        got = pr.round(None if r is None else to_np([r])[0])
        assert [tup(x) for x in got] == want, j
        r = rnd_f(rng)
    if rounds:
        ref.finalize(r)
        pr.finalize(to_np([r])[0])
        assert tup(pr.final_value()) == ref.final_value()


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_gkr_verifies_and_claimed_w_values(k):
    """The reference's run_gkr_test (src/provers/gkr.rs:215-272): the proof
    verifies against the direct sum, the final claim equals final_value, and
    claimed_w_values are W's multilinear extension at the b and c challenges."""
    rng = random.Random(k)
    add_, mult_, w = gkr_inputs(rng, k)
    n = 1 << k
    s = R.ZERO
    for b in range(n):
        for c in range(n):
            s = R.add(s, R.RefGkr.term(add_[b * n + c], mult_[b * n + c], w[b], w[c]))
    pr = O.Prover.gkr(1, np.array([x[0] for x in add_], np.uint64), np.array([x[0] for x in mult_], np.uint64),
                      np.array([x[0] for x in w], np.uint64))
    rp, ch, fv = O.sumcheck(pr, 2 * k, O.Transcript(1, label=b"gkr"))
    _, fc = O.verify(s, 2, 2 * k, O.Transcript(1, label=b"gkr"), rp)
    assert (fc == fv).all()
    wv = pr.claimed_w_values()
    pts = [tup(c) for c in ch]
    assert tup(wv[0]) == R.mle_eval_msb(w, pts[:k])
    assert tup(wv[1]) == R.mle_eval_msb(w, pts[k:])


def test_gkr_zero_gates_and_add_only():
    """src/provers/gkr.rs:281-345: zero gates give all-zero round polynomials;
    add-only circuits still prove the add sum."""
    rng = random.Random(99)
    k = 2
    add_, mult_, w = gkr_inputs(rng, k, zero_all=True)
    pr = O.Prover.gkr(3, to_np(add_), to_np(mult_), to_np(w))
    rp, _, _ = O.sumcheck(pr, 2 * k, O.Transcript(3, label=b"z"))
    assert not rp.any()
    add_, mult_, w = gkr_inputs(rng, k, zero_mult=True)
    n = 1 << k
    s = R.ZERO
    for b in range(n):
        for c in range(n):
            s = R.add(s, R.mul(add_[b * n + c], R.add(w[b], w[c])))
    pr = O.Prover.gkr(3, to_np(add_), to_np(mult_), to_np(w))
    rp, ch, fv = O.sumcheck(pr, 2 * k, O.Transcript(3, label=b"a"))
    _, fc = O.verify(s, 2, 2 * k, O.Transcript(3, label=b"a"), rp)
    assert (fc == fv).all()



# ---- protogalaxy::fold (src/folding.rs:14-75) ----------------------------------
def test_pg_fold_two_polys():
    """src/folding.rs:82-98: p0 = 1, p1 = X, (a, b) = (3, 5) gives
    (1 - a) + (a - b) X + b X^2."""
    r = O.protogalaxy_fold([(3, 5)], [[1], [0, 1]])
    assert [int(x) for x in r[:, 0]] == [(1 - 3) % O.P, (3 - 5) % O.P, 5]
    assert not r[:, 1:].any()


def test_pg_fold_four_polys():
    """src/folding.rs:100-114: constants 1..4 with (1, 0) at both levels
    select the last one."""
    r = O.protogalaxy_fold([(1, 0)] * 2, [[1], [2], [3], [4]])
    assert r.shape[0] == 1 and int(r[0, 0]) == 4


@pytest.mark.parametrize("n,deg,ext", [(8, 2, False), (16, 5, True), (32, 0, False), (2, 3, True)])
def test_pg_fold_matches_naive(n, deg, ext):
    """src/folding.rs:116-162: random polynomials of degree `deg`, log2 n
    levels, against the naive per-level polynomial arithmetic."""
    rng = random.Random(n * 31 + deg)
    el = (lambda: (rng.randrange(R.P), rng.randrange(R.P), rng.randrange(R.P))) if ext else \
        (lambda: (rng.randrange(R.P), 0, 0))
    polys = [[el() for _ in range(deg + 1)] for _ in range(n)]
    pairs = [(el(), el()) for _ in range(n.bit_length() - 1)]
    got = O.protogalaxy_fold(pairs, [np.array(p, dtype=np.uint64) for p in polys])
    want = R.protogalaxy_fold_naive(pairs, polys)
    assert [tuple(int(x) for x in row) for row in got] == want


def test_pg_fold_edges():
    P = O.P
    assert O.protogalaxy_fold([], []).shape[0] == 0                       # no polynomials: zero
    assert O.protogalaxy_fold([(1, 2)], [[5, 7, 0]]).tolist() == [[5, 0, 0], [7, 0, 0]]   # one: itself
    assert O.protogalaxy_fold([(1, 2)], [[0, 0]]).shape[0] == 0           # one zero polynomial
    assert O.protogalaxy_fold([(3, 4)], [[1], [1]]).tolist() == [[1, 0, 0]]  # zero difference: [p0], >= 1 term
    assert O.protogalaxy_fold([(3, 4)], [[], []]).tolist() == [[0, 0, 0]]
    # odd count: the last polynomial is dropped at the level it is left over
    a = O.protogalaxy_fold([(3, 4)], [[1], [2], [9]])
    b = O.protogalaxy_fold([(3, 4)], [[1], [2]])
    assert a.tolist() == b.tolist()
    # more levels than log2 n: the extra levels change nothing
    c = O.protogalaxy_fold([(3, 4), (5, 6), (7, 8)], [[1], [2]])
    assert c.tolist() == b.tolist()
    # fewer levels than log2 n: the result is the first of the remaining polynomials
    d = O.protogalaxy_fold([(3, 4)], [[1], [2], [10], [20]])
    assert d.tolist() == b.tolist()
    assert int(b[0, 0]) == (1 + 3 * (2 - 1)) % P and int(b[1, 0]) == 4
