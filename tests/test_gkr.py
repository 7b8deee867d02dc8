"""GkrProver (src/provers/gkr.rs) on the GPU: the witness kept as two compact
tables W_b, W_c instead of the reference's broadcast tables.  Every round
polynomial, challenge, final value and claimed W value must equal the
oracle's (which expands the broadcast tables exactly as the reference does),
for full, partial and over-long runs, through the per-round API and the
device-resident protocol."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def inputs(k, ext, seed):
    g = np.random.default_rng(seed)
    n = 1 << k
    shape = lambda m: (m, 3) if ext else (m,)  # noqa: E731
    return (g.integers(0, O.P, size=shape(n * n), dtype=np.uint64),
            g.integers(0, O.P, size=shape(n * n), dtype=np.uint64),
            g.integers(0, O.P, size=shape(n), dtype=np.uint64))


def check(E, proof, field, rp, ch, fv):
    n = rp.shape[0]
    assert np.array_equal(np.asarray(proof.round_polys).reshape(n, 2, field), rp[:, :, :field])
    assert np.array_equal(np.asarray(proof.challenges).reshape(n, field), ch[:, :field])
    assert np.array_equal(np.asarray(proof.final_value).reshape(field), fv[:field])


@pytest.mark.parametrize("k", [0, 1, 2, 3, 4, 6, 8])
@pytest.mark.parametrize("field,ext", [(1, False), (3, False), (3, True)])
@pytest.mark.parametrize("path", ["device_graph", "device", "host"])
def test_gkr_full_runs(E, k, field, ext, path):
    add, mult, w = inputs(k, ext, 10 * k + field + ext)
    rounds = 2 * k
    orc = O.Prover.gkr(field, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"gkr"), hook=bytes(range(32)))
    g = E.GkrProver(add, mult, w, field=field)
    if path == "host":
        proof = E.sumcheck(g, rounds, E.Transcript.keccak(field, b"gkr"),
                           hook=lambda r, t: t.absorb(bytes(range(32))))
    else:
        proof = g.prove(rounds, E.Transcript.keccak(field, b"gkr"), hook=bytes(range(32)),
                        use_graph=path == "device_graph")
    if rounds:
        check(E, proof, field, rp, ch, fv)
    cw = orc.claimed_w_values()
    assert np.array_equal(g.claimed_w_values(), cw[:, :field])


@pytest.mark.parametrize("k", [2, 3, 5])
@pytest.mark.parametrize("rounds_of", [lambda k: 1, lambda k: k, lambda k: k + 1, lambda k: 2 * k + 2])
def test_gkr_partial_and_extra_rounds(E, k, rounds_of):
    rounds = rounds_of(k)
    add, mult, w = inputs(k, False, 77 + k + rounds)
    orc = O.Prover.gkr(3, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(3, label=b"p"))
    g = E.GkrProver(add, mult, w)
    proof = g.prove(rounds, E.Transcript.keccak(3, b"p"))
    check(E, proof, 3, rp, ch, fv)
    assert np.array_equal(g.claimed_w_values(), orc.claimed_w_values())
    # add and mult after the run equal the oracle's tables
    for t in range(2):
        assert np.array_equal(g.table(t).reshape(-1, 3), orc.table(t))


def test_gkr_large_and_verifies(E):
    k = 10
    add, mult, w = inputs(k, False, 5)
    rounds = 2 * k
    orc = O.Prover.gkr(3, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(3, label=b"L"))
    g = E.GkrProver(add, mult, w)
    proof = g.prove(rounds, E.Transcript.keccak(3, b"L"))
    check(E, proof, 3, rp, ch, fv)
    g.reset()
    proof2 = g.prove(rounds, E.Transcript.keccak(3, b"L"))
    check(E, proof2, 3, rp, ch, fv)


def test_gkr_rejects(E):
    with pytest.raises(AssertionError):
        E.GkrProver(np.zeros(8, np.uint64), np.zeros(9, np.uint64), np.zeros(3, np.uint64))
    with pytest.raises(E.EffscError):      # |w| not a power of two
        E.GkrProver(np.zeros(9, np.uint64), np.zeros(9, np.uint64), np.zeros(3, np.uint64))


@pytest.mark.parametrize("k", [3, 4, 7])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("rounds_of", [lambda k: 3, lambda k: k + 1, lambda k: 2 * k])
@pytest.mark.parametrize("hook", [b"", b"\x05\x06\x07"])
def test_gkr_first_rounds_equal_per_round(E, k, field, rounds_of, hook):
    """Rounds 0-1 from one pass and round 2 from a double fold (base inputs,
    k >= 3) give the per-round path's proof, gate tables and claimed W values,
    and the oracle's proof."""
    rounds = rounds_of(k)
    add, mult, w = inputs(k, False, 900 + 7 * k + rounds + field + len(hook))
    p = E.GkrProver(add, mult, w, field=field)
    q = E.GkrProver(add, mult, w, field=field)
    q.set_first_rounds(False)
    for g in (p, q):
        g.set_tail(0)         # the one-block tail would take these sizes from round 0
    for use_graph in (True, False):
        p.reset()
        q.reset()
        x = p.prove(rounds, E.Transcript.keccak(field, b"g01"), hook=hook, use_graph=use_graph)
        y = q.prove(rounds, E.Transcript.keccak(field, b"g01"), hook=hook, use_graph=use_graph)
        assert np.array_equal(x.round_polys, y.round_polys)
        assert np.array_equal(x.challenges, y.challenges)
        assert np.array_equal(x.final_value, y.final_value)
        for t in range(2):
            assert np.array_equal(p.table(t), q.table(t))
        assert np.array_equal(p.claimed_w_values(), q.claimed_w_values())
    orc = O.Prover.gkr(field, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"g01"), hook=hook)
    check(E, x, field, rp, ch, fv)
    assert np.array_equal(p.claimed_w_values(), orc.claimed_w_values()[:, :field])


@pytest.mark.parametrize("field", [1, 3])
def test_gkr_runs_large(E, field):
    """k = 11: the rounds 0-1 pass, the round-2 pass and rounds 1, 3, 4 of the
    per-round path are large enough that lanes take runs of pairs sharing one
    W_b entry; proofs, gate tables after a partial run and claimed W values
    equal the per-pair forms' (the oracle's)."""
    k = 11
    add, mult, w = inputs(k, False, 4242 + field)
    orc = O.Prover.gkr(field, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, 2 * k, O.Transcript(field, label=b"runs"))
    for first in (True, False):
        g = E.GkrProver(add, mult, w, field=field)
        g.set_first_rounds(first)
        check(E, g.prove(2 * k, E.Transcript.keccak(field, b"runs")), field, rp, ch, fv)
        assert np.array_equal(g.claimed_w_values(), orc.claimed_w_values()[:, :field])
    part = O.Prover.gkr(field, add, mult, w)
    O.sumcheck(part, 5, O.Transcript(field, label=b"runs5"))
    g = E.GkrProver(add, mult, w, field=field)
    g.prove(5, E.Transcript.keccak(field, b"runs5"))
    for t in range(2):
        assert np.array_equal(g.table(t).reshape(-1, field), part.table(t)[:, :field])


@pytest.mark.parametrize("k", [1, 2, 3, 5, 6, 8])
@pytest.mark.parametrize("field,ext", [(1, False), (3, False), (3, True)])
@pytest.mark.parametrize("rounds_of", [lambda k: 1, lambda k: k, lambda k: 2 * k, lambda k: 2 * k + 2])
def test_gkr_tail_equals_per_round(E, k, field, ext, rounds_of):
    """The one-block tail (entered at round 0 for small k, mid-proof for
    k = 8) gives the per-round path's proof, all four tables after the run
    and claimed W values, and the oracle's proof."""
    rounds = rounds_of(k)
    hook = b"\x01\x02\x03" if k % 2 else bytes(range(16))
    add, mult, w = inputs(k, ext, 1300 + 11 * k + rounds + field + ext)
    p = E.GkrProver(add, mult, w, field=field)
    q = E.GkrProver(add, mult, w, field=field)
    q.set_tail(0)
    for use_graph in (True, False):
        p.reset()
        q.reset()
        x = p.prove(rounds, E.Transcript.keccak(field, b"gt"), hook=hook, use_graph=use_graph)
        y = q.prove(rounds, E.Transcript.keccak(field, b"gt"), hook=hook, use_graph=use_graph)
        assert np.array_equal(x.round_polys, y.round_polys)
        assert np.array_equal(x.challenges, y.challenges)
        assert np.array_equal(x.final_value, y.final_value)
        for t in range(4):
            assert np.array_equal(p.table(t), q.table(t)), t
        assert np.array_equal(p.claimed_w_values(), q.claimed_w_values())
    orc = O.Prover.gkr(field, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"gt"), hook=hook)
    check(E, x, field, rp, ch, fv)


def test_gkr_runs_k12_fp3(E):
    """k = 12 over Fp3 challenges with base gate tables (the bench size): the
    grid gives every lane four pairs, so the b-variable passes group runs of
    up to 16 pairs per W_b entry (g = 4..16) -- sizes the k = 11 case does
    not reach.  The proof and claimed W values equal the oracle's."""
    k = 12
    add, mult, w = inputs(k, False, 1212)
    orc = O.Prover.gkr(3, add, mult, w)
    rp, ch, fv = O.sumcheck(orc, 2 * k, O.Transcript(3, label=b"k12"))
    g = E.GkrProver(add, mult, w, field=3)
    check(E, g.prove(2 * k, E.Transcript.keccak(3, b"k12")), 3, rp, ch, fv)
    assert np.array_equal(g.claimed_w_values(), orc.claimed_w_values())
