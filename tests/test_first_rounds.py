"""InnerProduct rounds 0-2 in two passes (round 1 from base-field sums of
round 0's pass, round 2 folding with r0 and r1): proofs, challenges, final
values and post-state tables identical to one pass per round and to the
oracle, for full and partial runs, with and without hooks."""
import random

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def tables(n, seed):
    g = np.random.default_rng(seed)
    return [g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(2)]


@pytest.mark.parametrize("n", [3, 4, 5, 7, 10, 13, 16])
@pytest.mark.parametrize("hook", [b"", bytes(range(32)), b"\x05\x06\x07"])
@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_full_runs(E, n, hook, order):
    a, b = tables(n, 100 + n + len(hook))
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p = cls(a, b)
    p.set_tail(0)
    q = cls(a, b)
    q.set_tail(0)
    q.set_first_rounds(False)
    for use_graph in (True, True, False):
        p.reset()
        q.reset()
        x = p.prove(n, E.Transcript.keccak(3, b"fr"), hook=hook, use_graph=use_graph)
        y = q.prove(n, E.Transcript.keccak(3, b"fr"), hook=hook, use_graph=use_graph)
        assert np.array_equal(x.round_polys, y.round_polys)
        assert np.array_equal(x.challenges, y.challenges)
        assert np.array_equal(x.final_value, y.final_value)
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), n,
                            O.Transcript(3, label=b"fr"), hook=hook)
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.challenges, ch)
    assert np.array_equal(x.final_value, fv)


@pytest.mark.parametrize("rounds", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_partial_runs_post_state(E, rounds, order):
    n = 9
    a, b = tables(n, rounds)
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p = cls(a, b)
    p.set_tail(0)
    q = cls(a, b)
    q.set_tail(0)
    q.set_first_rounds(False)
    x = p.prove(rounds, E.Transcript.keccak(3, b"pr"), hook=bytes(range(32)))
    y = q.prove(rounds, E.Transcript.keccak(3, b"pr"), hook=bytes(range(32)))
    assert np.array_equal(x.round_polys, y.round_polys)
    assert np.array_equal(x.final_value, y.final_value)
    for t in range(2):
        assert np.array_equal(p.table(t), q.table(t))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), rounds,
                            O.Transcript(3, label=b"pr"), hook=bytes(range(32)))
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.final_value, fv)


@pytest.mark.parametrize("n", [17, 19])
@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("hook", [b"", b"\x05\x06\x07"])
def test_large_first_pass(E, n, order, hook):
    """Tables of 2^17 entries and more (multi-wave grids of the rounds 0-1
    pass and TMA-staged later rounds): proofs equal the per-round path's and
    the oracle's, for full and partial runs."""
    a, b = tables(n, 600 + n + len(hook))
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    for rounds in (3, n):
        p = cls(a, b)
        q = cls(a, b)
        q.set_first_rounds(False)
        x = p.prove(rounds, E.Transcript.keccak(3, b"tma01"), hook=hook)
        y = q.prove(rounds, E.Transcript.keccak(3, b"tma01"), hook=hook)
        assert np.array_equal(x.round_polys, y.round_polys)
        assert np.array_equal(x.challenges, y.challenges)
        assert np.array_equal(x.final_value, y.final_value)
        if rounds == 3:
            for t in range(2):
                assert np.array_equal(p.table(t), q.table(t))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), n,
                            O.Transcript(3, label=b"tma01"), hook=hook)
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.challenges, ch)
    assert np.array_equal(x.final_value, fv)


def test_default_path_large(E):
    """n = 20 with the default plan (two-pass start, TMA rounds, tail)."""
    n = 20
    a, b = tables(n, 7)
    x = E.InnerProductProver(a, b).prove(n, E.Transcript.keccak(3, b"big"))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB, 3, [a, b]), n, O.Transcript(3, label=b"big"))
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.final_value, fv)


@pytest.mark.parametrize("v", [4, 5, 9, 12, 15])
@pytest.mark.parametrize("extra", [0, 1, 99])
@pytest.mark.parametrize("field", [1, 3])
def test_eq_factored_left_phase_from_inner_sums(E, v, extra, field):
    """EqFactored runs that cover the left phase: the left rounds as
    InnerProduct rounds on (eq_l, inner sums) and p folded by the left
    challenges in one weighted pass give the per-round path's proof and
    post-state tables, and the oracle's."""
    rounds = min(v, v // 2 + extra)
    g = np.random.default_rng(300 + v + extra + field)
    w = g.integers(0, O.P, size=(v, 3) if field == 3 else v, dtype=np.uint64)
    p = g.integers(0, O.P, size=1 << v, dtype=np.uint64)
    fast = E.EqFactoredProver(w, p, field=field)
    slow = E.EqFactoredProver(w, p, field=field)
    slow.set_first_rounds(False)
    hook = bytes(range(32))
    x = fast.prove(rounds, E.Transcript.keccak(field, b"eqf"), hook=hook)
    y = slow.prove(rounds, E.Transcript.keccak(field, b"eqf"), hook=hook)
    assert np.array_equal(x.round_polys, y.round_polys)
    assert np.array_equal(x.challenges, y.challenges)
    assert np.array_equal(x.final_value, y.final_value)
    for t in range(3):
        assert np.array_equal(fast.table(t), slow.table(t))
    w3 = O.as_table(w)
    rp, ch, fv = O.sumcheck(O.Prover.eq_factored(field, w3, p), rounds, O.Transcript(field, label=b"eqf"), hook=hook)
    assert np.array_equal(np.asarray(x.round_polys).reshape(rounds, 2, field), rp[:, :, :field])
    assert np.array_equal(np.asarray(x.final_value).reshape(field), fv[:field])


# ---- Multilinear: rounds 0-1 from quarter sums, round 2 with a double fold ----
@pytest.mark.parametrize("n", [3, 4, 5, 7, 10, 13, 16])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("hook", [b"", bytes(range(32)), b"\x05\x06\x07"])
def test_ml_full_runs(E, n, field, hook):
    v = tables(n, 300 + n + field + len(hook))[0]
    p = E.MultilinearProver(v, field=field)
    p.set_tail(0)
    q = E.MultilinearProver(v, field=field)
    q.set_tail(0)
    q.set_first_rounds(False)
    for use_graph in (True, False):
        p.reset()
        q.reset()
        x = p.prove(n, E.Transcript.keccak(field, b"mlfr"), hook=hook, use_graph=use_graph)
        y = q.prove(n, E.Transcript.keccak(field, b"mlfr"), hook=hook, use_graph=use_graph)
        assert np.array_equal(x.round_polys, y.round_polys)
        assert np.array_equal(x.challenges, y.challenges)
        assert np.array_equal(x.final_value, y.final_value)
    rp, ch, fv = O.sumcheck(O.Prover(O.ML, O.MSB, field, [v]), n, O.Transcript(field, label=b"mlfr"), hook=hook)
    assert np.array_equal(np.asarray(x.round_polys).reshape(n, 1, field), rp[:, :1, :field])
    assert np.array_equal(np.asarray(x.challenges).reshape(n, field), ch[:, :field])
    assert np.array_equal(np.asarray(x.final_value).reshape(field), fv[:field])


@pytest.mark.parametrize("n", [18, 20])
def test_ml_default_schedule(E, n):
    """Two-pass start, multi-block rounds, cluster tail and one-block tail in
    one proof, as the default schedule runs them."""
    v = tables(n, 400 + n)[0]
    pf = E.MultilinearProver(v, field=1).prove(n, E.Transcript.keccak(1, b"mlds"))
    rp, ch, fv = O.sumcheck(O.Prover(O.ML, O.MSB, 1, [v]), n, O.Transcript(1, label=b"mlds"))
    assert np.array_equal(np.asarray(pf.round_polys).reshape(n, 1, 1), rp[:, :1, :1])
    assert np.array_equal(np.asarray(pf.final_value).reshape(1), fv[:1])


@pytest.mark.parametrize("rounds", [3, 4, 6])
@pytest.mark.parametrize("field", [1, 3])
def test_ml_partial_post_state(E, rounds, field):
    n = 9
    v = tables(n, 500 + rounds + field)[0]
    p = E.MultilinearProver(v, field=field)
    p.set_tail(0)
    pf = p.prove(rounds, E.Transcript.keccak(field, b"mlpart"))
    orc = O.Prover(O.ML, O.MSB, field, [v])
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"mlpart"))
    assert np.array_equal(np.asarray(pf.round_polys).reshape(rounds, 1, field), rp[:, :1, :field])
    got = np.asarray(p.table(0)).reshape(-1, field)
    assert np.array_equal(got, orc.table(0)[:, :field])


# ---- InnerProduct rounds 0-3 in two passes (26 interpolation sums, triple fold) ----
@pytest.mark.parametrize("n", [14, 15, 17, 19])
@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("hook", [b"", b"\x05\x06\x07", bytes(range(32))])
def test_rounds_0_3_two_passes(E, n, order, hook):
    """The three-round start gives the two-pass start's and the per-round
    path's proofs and post-state tables (full and partial runs, graph and
    direct launches) and the oracle's proof."""
    a, b = tables(n, 800 + n + len(hook))
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    for rounds in (4, 5, n):
        provers = []
        for level in (2, 1, 0):
            p = cls(a, b)
            p.set_first_rounds(level)
            provers.append(p)
        for use_graph in (True, False):
            proofs = []
            for p in provers:
                p.reset()
                proofs.append(p.prove(rounds, E.Transcript.keccak(3, b"r03"), hook=hook, use_graph=use_graph))
            for y in proofs[1:]:
                assert np.array_equal(proofs[0].round_polys, y.round_polys)
                assert np.array_equal(proofs[0].challenges, y.challenges)
                assert np.array_equal(proofs[0].final_value, y.final_value)
            if rounds < n:
                for t in range(2):
                    for q in provers[1:]:
                        assert np.array_equal(provers[0].table(t), q.table(t))
        rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), rounds,
                                O.Transcript(3, label=b"r03"), hook=hook)
        assert np.array_equal(proofs[0].round_polys, rp)
        assert np.array_equal(proofs[0].challenges, ch)
        assert np.array_equal(proofs[0].final_value, fv)


@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_rounds_0_3_edge_values(E, order):
    """Tables of the extreme canonical values 0, 1, p - 1 and 2^32 (every
    difference and interpolation sum wraps): the three-round start equals the
    oracle."""
    n = 14
    g = np.random.default_rng(4)
    pick = np.array([0, 1, O.P - 1, 1 << 32, O.P - 2, (1 << 32) - 1], dtype=np.uint64)
    a = pick[g.integers(0, pick.size, size=1 << n)]
    b = pick[g.integers(0, pick.size, size=1 << n)]
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    x = cls(a, b).prove(n, E.Transcript.keccak(3, b"edge"))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), n,
                            O.Transcript(3, label=b"edge"))
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.final_value, fv)
