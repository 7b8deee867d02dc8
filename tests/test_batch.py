"""Batched proving (effsc_batch_*): a cohort of independent InnerProduct /
Multilinear MSB provers of uneven size proved with one kernel per round.

Every instance's proof must be bit-identical to the oracle's proof of that
instance alone (runner::sumcheck, src/runner.rs:29-69, all rounds, Keccak
transcript labelled per instance, no hook) and to the single-instance GPU
path, with and without graph replay, before and after autotuning."""
import json
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


def label(i):
    return ("effsc-gpu/batch/%d" % i).encode()


def oracle_proof(kind, field, tabs, n, lab):
    pr = O.Prover(O.IP if kind == "ip" else O.ML, O.MSB, field, tabs)
    return O.sumcheck(pr, n, O.Transcript(field, label=lab))


def check_against_oracle(kind, field, nv, tabs, proofs):
    for i, n in enumerate(nv):
        rp, ch, fv = oracle_proof(kind, field, tabs[i], n, label(i))
        p = proofs[i]
        assert np.array_equal(np.asarray(p.round_polys).reshape(n, -1, field), rp[:, :, :field].reshape(n, -1, field)), i
        assert np.array_equal(np.asarray(p.challenges).reshape(n, field), ch[:, :field]), i
        assert np.array_equal(np.asarray(p.final_value).reshape(field), fv[:field]), i


def make_tabs(rng, kind, nv):
    ntab = 2 if kind == "ip" else 1
    out = []
    for n in nv:
        g = np.random.default_rng(rng.randrange(1 << 62))
        out.append([g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(ntab)])
    return out


def transcripts(E, field, n):
    return [E.Transcript.keccak(field, label(i)) for i in range(n)]


@pytest.mark.parametrize("kind", ["ip", "ml"])
@pytest.mark.parametrize("field", [1, 3])
def test_batch_matches_oracle(E, kind, field):
    rng = random.Random(1000 + 10 * field + (kind == "ip"))
    nv = [1, 2, 3, 5, 8, 11, 4, 1, 12, 7, 9, 2, 10, 6, 13, 3]
    tabs = make_tabs(rng, kind, nv)
    b = E.Batch(E.IP if kind == "ip" else E.ML, nv, tables=tabs, field=field)
    for use_graph in (True, False, True):
        proofs = b.prove(transcripts(E, field, len(nv)), use_graph=use_graph)
        check_against_oracle(kind, field, nv, tabs, proofs)


@pytest.mark.parametrize("q", [1, 3, 8, 64])
def test_batch_granularity(E, q):
    rng = random.Random(77 + q)
    nv = [14, 3, 9, 12, 1, 15]
    tabs = make_tabs(rng, "ip", nv)
    b = E.Batch(E.IP, nv, tables=tabs, field=3)
    b.set_quads_per_thread(q)
    check_against_oracle("ip", 3, nv, tabs, b.prove(transcripts(E, 3, len(nv))))


def test_batch_equals_single_path(E):
    """A 64-instance cohort with seeded device tables (num_vars 1..16) against
    the single-instance device path, instance by instance."""
    rng = random.Random(4242)
    nv = [rng.randint(1, 16) for _ in range(64)]
    seeds = [[0xBA7C0000 + 2 * i, 0xBA7C0000 + 2 * i + 1] for i in range(64)]
    b = E.Batch(E.IP, nv, seeds=seeds, field=3)
    proofs = b.prove(transcripts(E, 3, len(nv)))
    for i, n in enumerate(nv):
        a = E.gen_uniform(seeds[i][0], 1 << n)
        bb = E.gen_uniform(seeds[i][1], 1 << n)
        solo = E.InnerProductProver(a, bb, field=3).prove(n, E.Transcript.keccak(3, label(i)))
        assert np.array_equal(solo.round_polys, proofs[i].round_polys), i
        assert np.array_equal(solo.challenges, proofs[i].challenges), i
        assert np.array_equal(solo.final_value, proofs[i].final_value), i
    # spot-check a few against the oracle directly
    for i in range(0, 64, 13):
        n = nv[i]
        tabs = [O.gen_table(seeds[i][0], 1 << n), O.gen_table(seeds[i][1], 1 << n)]
        rp, ch, fv = oracle_proof("ip", 3, tabs, n, label(i))
        assert np.array_equal(proofs[i].round_polys, rp), i
        assert np.array_equal(proofs[i].final_value, fv), i


def test_batch_tune_persists(E, tmp_path):
    rng = random.Random(9)
    nv = [rng.randint(4, 14) for _ in range(24)]
    tabs = make_tabs(rng, "ip", nv)
    b = E.Batch(E.IP, nv, tables=tabs, field=3)
    path = str(tmp_path / "tune.jsonl")
    q, tail = b.tune(transcripts(E, 3, len(nv)), cache_path=path)
    assert q in (1, 2, 4, 8)
    assert tail in (0, 1 << 6, 1 << 8, 1 << 10, (1 << 64) - 1)
    rec = json.loads(open(path).read().strip().splitlines()[-1])
    assert rec["quads_per_thread"] == q and rec["instances"] == len(nv) and len(rec["ms"]) == 20
    check_against_oracle("ip", 3, nv, tabs, b.prove(transcripts(E, 3, len(nv))))


@pytest.mark.parametrize("kind", ["ip", "ml"])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("tail", [0, 4, 8, 64, 1 << 10, None])
def test_batch_tail_switch(E, kind, field, tail):
    """Every tail switch point gives the same proofs; instances smaller than
    the switch run entirely in the tail kernel."""
    rng = random.Random(31 + field + (tail or 0) % 97)
    nv = [1, 2, 3, 4, 6, 9, 12, 14, 5, 2, 11]
    tabs = make_tabs(rng, kind, nv)
    b = E.Batch(E.IP if kind == "ip" else E.ML, nv, tables=tabs, field=field)
    b.set_tail(tail)
    check_against_oracle(kind, field, nv, tabs, b.prove(transcripts(E, field, len(nv))))


def test_batch_launches_one_kernel_per_round(E):
    nv = [3, 6, 2, 6]
    rng = random.Random(5)
    b = E.Batch(E.ML, nv, tables=make_tabs(rng, "ml", nv), field=3)
    b.set_tail(0)
    b.prove_raw(transcripts(E, 3, len(nv)))
    E.launch_count_reset()
    b.prove_raw(transcripts(E, 3, len(nv)))
    assert E.launch_count() == max(nv) + 1     # one per round + one final fold
    b.set_tail(8)                              # rounds on tables of <= 8 entries: one tail launch
    b.prove_raw(transcripts(E, 3, len(nv)))
    E.launch_count_reset()
    b.prove_raw(transcripts(E, 3, len(nv)))
    assert E.launch_count() == (6 - 3 + 1) + 1 + 1


def test_batch_rejects_bad_input(E):
    with pytest.raises(E.EffscError):
        E.Batch(E.IP, [0], seeds=[[1, 2]])
    with pytest.raises(E.EffscError):
        E.Batch(E.COEF, [4], seeds=[[1]])
    b = E.Batch(E.IP, [4, 5], seeds=[[1, 2], [3, 4]])
    with pytest.raises(ValueError):
        b.prove([E.Transcript.keccak(3, b"x")])
    with pytest.raises(E.EffscError):
        b.prove([E.Transcript.keccak(1, b"x"), E.Transcript.keccak(3, b"y")])
    with pytest.raises(E.EffscError):
        b.set_quads_per_thread(0)
