"""The one-block tail kernel of effsc_prove (Multilinear / InnerProduct, MSB and LSB):
proofs and post-states identical to the per-round path and to the oracle for
every switch point, field, partial run and hook."""
import random
import zlib

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

HOOK = bytes(range(32))


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def make(E, kind, field, n, rng):
    g = np.random.default_rng(rng.randrange(1 << 62))
    tabs = [g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(2 if kind == "ip" else 1)]
    if kind == "ip":
        return tabs, E.InnerProductProver(tabs[0], tabs[1], field=field)
    return tabs, E.MultilinearProver(tabs[0], field=field)


@pytest.mark.parametrize("kind", ["ip", "ml"])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 12, 15])
@pytest.mark.parametrize("tail", [4, 64, None])
def test_tail_full_proof(E, kind, field, n, tail):
    rng = random.Random(zlib.crc32(b"%s/%d/%d" % (kind.encode(), field, n)))
    tabs, p = make(E, kind, field, n, rng)
    p.set_tail(tail)
    label = b"effsc-gpu/tail/%d" % n
    for use_graph in (True, True, False):
        p.reset()
        pf = p.prove(n, E.Transcript.keccak(field, label), use_graph=use_graph)
        rp, ch, fv = O.sumcheck(O.Prover(O.IP if kind == "ip" else O.ML, O.MSB, field, tabs), n,
                                O.Transcript(field, label=label))
        assert np.array_equal(pf.round_polys.reshape(n, -1, field), rp[:, :, :field])
        assert np.array_equal(pf.challenges.reshape(n, field), ch[:, :field])
        assert np.array_equal(pf.final_value.reshape(field), fv[:field])


@pytest.mark.parametrize("kind", ["ip", "ml"])
@pytest.mark.parametrize("rounds", [1, 3, 7, 9])
def test_tail_partial_with_hook_matches_per_round_path(E, kind, rounds):
    """Partial runs with a hook: the tail must leave the same tables as the
    per-round kernels (post-state accessors), and the same proof."""
    n = 10
    rng = random.Random(rounds)
    tabs, p = make(E, kind, 3, n, rng)
    _, q = make(E, kind, 3, n, random.Random(rounds))
    p.set_tail(None)
    q.set_tail(0)
    a = p.prove(rounds, E.Transcript.keccak(3, b"t"), hook=HOOK)
    b = q.prove(rounds, E.Transcript.keccak(3, b"t"), hook=HOOK)
    assert np.array_equal(a.round_polys, b.round_polys)
    assert np.array_equal(a.challenges, b.challenges)
    assert np.array_equal(a.final_value, b.final_value)
    for t in range(len(tabs)):
        assert np.array_equal(p.table(t), q.table(t))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP if kind == "ip" else O.ML, O.MSB, 3, tabs), rounds,
                            O.Transcript(3, label=b"t"), hook=HOOK)
    assert np.array_equal(a.round_polys, rp)
    assert np.array_equal(a.final_value, fv)


def test_tail_cuts_launches(E):
    rng = random.Random(3)
    _, p = make(E, "ip", 3, 12, rng)
    p.set_tail(0)
    p.prove(12, E.Transcript.keccak(3, b"x"), use_graph=False)
    p.reset()
    E.launch_count_reset()
    p.prove(12, E.Transcript.keccak(3, b"x"), use_graph=False)
    per_round = E.launch_count()
    p.reset()
    p.set_tail(None)
    E.launch_count_reset()
    p.prove(12, E.Transcript.keccak(3, b"x"), use_graph=False)
    assert E.launch_count() < per_round


@pytest.mark.parametrize("hook_len", [1, 7, 8, 13, 40, 136, 137, 300])
@pytest.mark.parametrize("tail", [0, None])
def test_hook_lengths(E, hook_len, tail):
    """Hook bytes of every alignment and across the 136-byte rate: the word
    and byte forms of the device transcript agree with the oracle."""
    rng = random.Random(hook_len)
    tabs, p = make(E, "ip", 3, 8, rng)
    p.set_tail(tail)
    hook = bytes((7 * i + hook_len) & 0xFF for i in range(hook_len))
    pf = p.prove(8, E.Transcript.keccak(3, b"h"), hook=hook)
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB, 3, tabs), 8, O.Transcript(3, label=b"h"), hook=hook)
    assert np.array_equal(pf.round_polys, rp)
    assert np.array_equal(pf.challenges, ch)
    assert np.array_equal(pf.final_value, fv)


@pytest.mark.parametrize("kind", ["ml", "ip"])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("n,rounds", [(6, 6), (9, 4), (11, 7), (12, 12)])
def test_lsb_tail_proof_and_post_state(E, kind, field, n, rounds):
    """LSB provers run their tail on a bit-reversed shared-memory layout: the
    proof, the tables left after the runner's finalize and the final value
    equal the oracle's, full and partial runs, with a hook."""
    g = np.random.default_rng(1000 + n * 7 + rounds + field)
    k = 2 if kind == "ip" else 1
    tabs = [g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(k)]
    cls = E.InnerProductProverLSB if kind == "ip" else E.MultilinearProverLSB
    p = cls(*tabs, field=field)
    hook = bytes(range(24))
    pf = p.prove(rounds, E.Transcript.keccak(field, b"lsbtail"), hook=hook)
    orc = O.Prover(O.IP if kind == "ip" else O.ML, O.LSB, field, tabs)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"lsbtail"), hook=hook)
    assert np.array_equal(np.asarray(pf.round_polys).reshape(rounds, k, field), rp[:, :k, :field])
    assert np.array_equal(np.asarray(pf.challenges).reshape(rounds, field), ch[:, :field])
    assert np.array_equal(np.asarray(pf.final_value).reshape(field), fv[:field])
    for t in range(k):
        assert np.array_equal(np.asarray(p.table(t)).reshape(-1, field), orc.table(t)[:, :field]), t
