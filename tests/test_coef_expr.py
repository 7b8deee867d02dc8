"""CoefficientProver[LSB] with a declarative evaluator and tablewise tables,
and the legacy coefficient_sumcheck runner, against the big-integer
restatement with the reference's own test evaluators as callbacks
(coef_expr_ref.py; src/coefficient_sumcheck.rs:379-430).

CPU: the declarative form of each evaluator adds what its callback adds, on
random pairs.  GPU: proofs (per-round runner and device protocol), the
tables after the run and final_value equal the restatement's; the legacy
runner sends the first `degree` coefficients and reduces every round."""
import random
import zlib

import numpy as np
import pytest

import bigint_ref as R
import coef_expr_ref as C
from oracle import oracle as O

P = R.P


class _FakeE:
    """The factor helpers and Evaluator of effsc_gpu without loading it."""

    @staticmethod
    def pw_even(i):
        return ("pw", i, 0, 0)

    @staticmethod
    def pw_odd(i):
        return ("pw", i, 0, 1)

    @staticmethod
    def tw_even(t, c):
        return ("tw", t, c, 0)

    @staticmethod
    def tw_odd(t, c):
        return ("tw", t, c, 1)

    class Evaluator:
        def __init__(self, degree, terms):
            self.deg, self.terms = degree, terms


def run_declarative(ev, coeffs, tw, pw):
    for c, k, fs in ev.terms:
        p = R.lift(k) if isinstance(k, int) else tuple(k)
        for kind, t, col, odd in fs:
            x = pw[t][odd] if kind == "pw" else tw[t][odd][col]
            p = R.mul(p, x)
        coeffs[c] = R.add(coeffs[c], p)


@pytest.mark.parametrize("name", sorted(C.EVALUATORS))
def test_declarative_form_matches_callback(name):
    rng = random.Random(zlib.crc32(name.encode()))
    cb, deg = C.EVALUATORS[name]
    ev = C.declarative(_FakeE, name)
    el = lambda: (rng.randrange(P), rng.randrange(P), rng.randrange(P))  # noqa: E731
    for _ in range(50):
        pw = [(el(), el()), (el(), el())]
        tw = [([el(), el()], [el(), el()])]
        a, b = [R.ZERO] * (deg + 1), [R.ZERO] * (deg + 1)
        cb(a, tw, pw)
        run_declarative(ev, b, tw, pw)
        assert a == b


# ---------------------------------------------------------------------------
def setup_tables(name, n, field, rng):
    def rnd():
        return rng.randrange(P)
    shape = (n,) if field == 1 else (n, 3)
    pw_count = 2 if name == "inner_product" else 1
    pw = [np.array([rnd() for _ in range(int(np.prod(shape)))], dtype=np.uint64).reshape(shape)
          for _ in range(pw_count)]
    tw = []
    if name == "mixed":
        tshape = (n, 2) if field == 1 else (n, 2, 3)
        tw = [np.array([rnd() for _ in range(int(np.prod(tshape)))], dtype=np.uint64).reshape(tshape)]
    return pw, tw


def to_ref(x, field):
    a = np.asarray(x, dtype=np.uint64)
    if field == 1:
        return [int(v) for v in a.reshape(-1)] if a.ndim == 1 else [[int(v) for v in row] for row in a]
    if a.ndim == 2:
        return [tuple(int(v) for v in e) for e in a]
    return [[tuple(int(v) for v in e) for e in row] for row in a]


def ref_proof(name, order, pw, tw, field, rounds, label):
    """The restatement's proof; final value None where the reference panics."""
    cb, deg = C.EVALUATORS[name]
    ref = C.RefCoefProver(order, cb, deg, [to_ref(t, field) for t in tw], [to_ref(t, field) for t in pw])
    tr = O.Transcript(field, label=label)
    wires, chals, prev = [], [], None
    for _ in range(rounds):
        wire, _ = ref.round(prev)
        for v in wire:
            tr.send(np.array(v, dtype=np.uint64))
        wires.append(wire)
        prev = tuple(int(v) for v in tr.challenge())
        chals.append(prev)
    if prev is not None:
        ref.finalize(prev)
    try:
        fv = ref.final_value()
    except C.RefPanic:
        fv = None
    return ref, wires, chals, fv


def gpu_rounds(E, g, rounds, t):
    """The runner without final_value (src/runner.rs:39-60)."""
    rps, chs, prev = [], [], None
    for _ in range(rounds):
        ev = g.round(prev)
        for v in ev:
            t.send(v)
        rps.append(ev)
        prev = t.challenge()
        chs.append(prev)
    if prev is not None:
        g.finalize(prev)
    return np.array(rps), np.array(chs)


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(C.EVALUATORS))
@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("path", ["host", "device"])
def test_declarative_prover(E, name, order, field, path):
    rng = random.Random(len(name) * 100 + (order == "lsb") * 10 + field + (path == "device") * 1000)
    n = 1 << 6
    pw, tw = setup_tables(name, n, field, rng)
    rounds = 6 if path == "device" else 4
    ev = C.declarative(E, name)
    cls = E.CoefficientProver if order == "msb" else E.CoefficientProverLSB
    g = cls(pw, field=field, evaluator=ev, tablewise=tw)
    t = E.Transcript.keccak(field, b"expr")
    ref, wires, chals, fv = ref_proof(name, order, pw, tw, field, rounds, b"expr")
    if path == "host":
        # the runner's rounds, then final_value on its own: it panics where
        # the reference's does (mixed reads a tablewise row of a table that
        # still holds several rows)
        rp, ch = gpu_rounds(E, g, rounds, t)
        if fv is None:
            with pytest.raises(E.ReferencePanic):
                g.final_value()
        else:
            got_fv = g.final_value()
    else:
        pf = g.prove(rounds, t)
        rp, ch, got_fv = pf.round_polys, pf.challenges, pf.final_value
        assert fv is not None
    d = max(1, C.EVALUATORS[name][1])
    want_rp = np.array([[list(v)[:field] for v in w] for w in wires], dtype=np.uint64).reshape(rounds, d, field)
    assert np.array_equal(np.asarray(rp).reshape(rounds, d, field), want_rp)
    assert np.array_equal(np.asarray(ch).reshape(rounds, field),
                          np.array([list(c)[:field] for c in chals], dtype=np.uint64))
    if fv is not None:
        assert np.array_equal(np.asarray(got_fv).reshape(field), np.array(list(fv)[:field], dtype=np.uint64))
    # tables after the run: pairwise tables, then the tablewise columns
    cols = [t_ for t_ in ref.pw] + [[row[c] for row in t_] for t_ in ref.tw for c in range(len(t_[0]) if t_ else 0)]
    for i, col in enumerate(cols):
        got = np.asarray(g.table(i)).reshape(-1, field)
        assert np.array_equal(got, np.array([list(x)[:field] for x in col], dtype=np.uint64).reshape(-1, field)), i


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(C.EVALUATORS))
@pytest.mark.parametrize("field", [1, 3])
def test_legacy_coefficient_sumcheck(E, name, field):
    """src/coefficient_sumcheck.rs:255-365: LSB pairs, the first `degree`
    coefficients sent per round, every table reduced after each challenge."""
    rng = random.Random(7 + len(name) + field)
    n = 1 << 5
    pw, tw = setup_tables(name, n, field, rng)
    rounds = 4
    ev = C.declarative(E, name)
    res, prover = E.coefficient_sumcheck(ev, tw, pw, rounds, E.Transcript.keccak(field, b"legacy-coef"), field=field)
    cb, deg = C.EVALUATORS[name]
    ref = C.RefCoefProver("lsb", cb, deg, [to_ref(t, field) for t in tw], [to_ref(t, field) for t in pw])
    tr = O.Transcript(field, label=b"legacy-coef")
    for r in range(rounds):
        coeffs = ref.coefficients()
        for cf in coeffs[:deg]:
            tr.send(np.array(cf, dtype=np.uint64))
        ch = tuple(int(v) for v in tr.challenge())
        got = np.asarray(res.prover_messages[r]).reshape(-1, field)
        assert got.shape[0] == deg + 1
        assert np.array_equal(got, np.array([list(c)[:field] for c in coeffs], dtype=np.uint64))
        assert np.array_equal(np.asarray(res.verifier_messages[r]).reshape(field), np.array(ch[:field], dtype=np.uint64))
        ref.reduce(ch)
    for i, col in enumerate([t_ for t_ in ref.pw] + [[row[c] for row in t_] for t_ in ref.tw for c in range(2)]):
        got = np.asarray(prover.table(i)).reshape(-1, field)
        assert np.array_equal(got, np.array([list(x)[:field] for x in col], dtype=np.uint64).reshape(-1, field))


@pytest.mark.gpu
def test_declarative_rejects(E):
    v = np.arange(8, dtype=np.uint64)
    with pytest.raises(E.EffscError):      # five columns
        E.CoefficientProver([v, v, v, v, v], field=1, evaluator=E.Evaluator(1, [(0, 1, [E.pw_even(4)])]))
    with pytest.raises(E.EffscError):      # degree 4
        E.CoefficientProver([v], field=1, evaluator=E.Evaluator(4, [(0, 1, [E.pw_even(0)])]))
    with pytest.raises(E.EffscError):      # a factor on a column that does not exist
        E.CoefficientProver([v], field=1, evaluator=E.Evaluator(1, [(0, 1, [E.pw_even(1)])]))
