"""The Montgomery boundary across the drop-in surface.

The crate's field elements are arkworks Montgomery residues (x 2^64 mod p,
reference src/field.rs:314-375) and the Rust binding passes them as they lie
in memory with repr = EFFSC_MONTGOMERY.  Every prover kind in both orders and
both fields, through the per-round ABI (the host runner) and through
effsc_prove, is fed Montgomery inputs and a Montgomery transcript; every
output -- round polynomials, challenges, final value, the tables read back
after full and partial runs, final_evaluations, final_factors,
claimed_w_values -- is converted back to canonical form and must equal the
oracle's values on the canonical inputs.  effsc_fold and
effsc_build_eq_table likewise."""
import random
import zlib

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

P = O.P
R = (1 << 64) % P
RINV = pow(R, -1, P)


def _conv(x, f):
    a = np.asarray(x, dtype=np.uint64)
    flat = [int(v) * f % P for v in a.reshape(-1)]
    return np.array(flat, dtype=np.uint64).reshape(a.shape)


def mont(x):
    return _conv(x, R)


def canon(x):
    return _conv(x, RINV)


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def rand(rng, shape):
    return np.array([rng.randrange(P) for _ in range(int(np.prod(shape)))], dtype=np.uint64).reshape(shape)


def tables_for(kind, field, n, rng):
    shape = (n,) if field == 1 else (n, 3)
    if kind == "ml":
        return [rand(rng, shape)]
    if kind == "ip":
        return [rand(rng, shape), rand(rng, shape)]
    return [rand(rng, shape) for _ in range(3)]   # coefficient: eq-like, f, g


def make_gpu(E, kind, order, field, tabs, repr):
    msb = order == "msb"
    if kind == "ml":
        cls = E.MultilinearProver if msb else E.MultilinearProverLSB
        return cls(tabs[0], field=field, repr=repr)
    if kind == "ip":
        cls = E.InnerProductProver if msb else E.InnerProductProverLSB
        return cls(tabs[0], tabs[1], field=field, repr=repr)
    cls = E.CoefficientProver if msb else E.CoefficientProverLSB
    return cls(tabs, field=field, repr=repr)


def make_oracle(kind, order, tabs):
    k = {"ml": O.ML, "ip": O.IP, "coef": O.COEF}[kind]
    deg = {"ml": 1, "ip": 2, "coef": 3}[kind]
    return O.Prover(k, O.MSB if order == "msb" else O.LSB, deg, tabs)


def run(E, prover, field, rounds, path, repr):
    t = E.Transcript.keccak(field, b"mont", repr=repr)
    if path == "host":
        return E.sumcheck(prover, rounds, t)
    return prover.prove(rounds, t)


def check_against_oracle(pf, rp, ch, fv, field, d):
    rounds = rp.shape[0]
    assert np.array_equal(canon(pf.round_polys).reshape(rounds, d, field), rp[:, :d, :field])
    assert np.array_equal(canon(pf.challenges).reshape(rounds, field), ch[:, :field])
    assert np.array_equal(canon(pf.final_value).reshape(field), fv[:field])


@pytest.mark.parametrize("kind", ["ml", "ip", "coef"])
@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("path", ["host", "device"])
@pytest.mark.parametrize("full", [True, False])
def test_provers_montgomery(E, kind, order, field, path, full):
    rng = random.Random(zlib.crc32(repr((kind, order, field, path, full)).encode()))
    nv = 7
    n = 1 << nv
    tabs = tables_for(kind, field, n, rng)
    rounds = nv if full else 3
    g = make_gpu(E, kind, order, field, [mont(t) for t in tabs], E.MONTGOMERY)
    pf = run(E, g, field, rounds, path, E.MONTGOMERY)
    orc = make_oracle(kind, order, tabs)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"mont"))
    d = orc.degree()
    check_against_oracle(pf, rp, ch, fv, field, d)
    for i in range(len(tabs)):
        got = canon(g.table(i)).reshape(-1, field)
        assert np.array_equal(got, orc.table(i)[:, :field]), i
    if kind == "ip" and full:
        ea, eb = g.final_evaluations()
        assert np.array_equal(canon(ea).reshape(field), orc.table(0)[0, :field])
        assert np.array_equal(canon(eb).reshape(field), orc.table(1)[0, :field])


@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("path", ["host", "device"])
@pytest.mark.parametrize("rounds_of", [lambda v: v, lambda v: v // 2 + 1])
def test_eq_factored_montgomery(E, field, path, rounds_of):
    rng = random.Random(31 + field)
    v = 8
    w = rand(rng, (v,) if field == 1 else (v, 3))
    p = rand(rng, (1 << v,) if field == 1 else (1 << v, 3))
    rounds = rounds_of(v)
    g = E.EqFactoredProver(mont(w), mont(p), field=field, repr=E.MONTGOMERY)
    pf = run(E, g, field, rounds, path, E.MONTGOMERY)
    orc = O.Prover.eq_factored(field, O.as_table(w), p)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"mont"))
    check_against_oracle(pf, rp, ch, fv, field, 2)
    for i in range(3):
        assert np.array_equal(canon(g.table(i)).reshape(-1, field), orc.table(i)[:, :field]), i
    if rounds == v:
        p0, e = g.final_factors()
        assert np.array_equal(canon(p0).reshape(field), orc.table(0)[0, :field])
        want_e = O.f3_mul(orc.table(1)[0], orc.table(2)[0])
        assert np.array_equal(canon(e).reshape(field), want_e[:field])


@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("path", ["host", "device"])
def test_gkr_montgomery(E, field, path):
    rng = random.Random(77 + field)
    k = 3
    n = 1 << k
    shape = (lambda m: (m,)) if field == 1 else (lambda m: (m, 3))
    add, mult, w = rand(rng, shape(n * n)), rand(rng, shape(n * n)), rand(rng, shape(n))
    g = E.GkrProver(mont(add), mont(mult), mont(w), field=field, repr=E.MONTGOMERY)
    pf = run(E, g, field, 2 * k, path, E.MONTGOMERY)
    orc = O.Prover.gkr(field, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, 2 * k, O.Transcript(field, label=b"mont"))
    check_against_oracle(pf, rp, ch, fv, field, 2)
    assert np.array_equal(canon(g.claimed_w_values()).reshape(2, field), orc.claimed_w_values()[:, :field])


@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("n", [1, 7, 64, 1000])
def test_fold_montgomery(E, field, n):
    rng = random.Random(n * 3 + field)
    v = rand(rng, (n,) if field == 1 else (n, 3))
    w = [rng.randrange(P) for _ in range(field)]
    out = E.fold(mont(v), mont(np.array(w, dtype=np.uint64)), field=field, repr=E.MONTGOMERY)
    orc = O.Prover(O.ML, O.MSB, field, [v])
    orc.finalize(w + [0] * (3 - field))
    assert np.array_equal(canon(out).reshape(-1, field), orc.table(0)[:, :field])


@pytest.mark.parametrize("field", [1, 3])
def test_build_eq_table_montgomery(E, field):
    rng = random.Random(5 + field)
    v = 6
    w = rand(rng, (v,) if field == 1 else (v, 3))
    got = E.build_eq_table(mont(w), field=field, repr=E.MONTGOMERY)
    want = O.build_eq_table(O.as_table(w))
    assert np.array_equal(canon(got).reshape(-1, field), want[:, :field])
