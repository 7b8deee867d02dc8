"""Serving (effsc_server_*): continuous batching under an HBM budget.

Each proof must be the same whether the request is proved alone, through the
server alone, or in a mix of requests of other kinds, sizes and rounds that
were admitted while it was in flight -- and equal to the oracle's proof."""
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
    return b"effsc-gpu/serve/%d" % i


def workload(seed, count, lo, hi, ml_frac=0.3):
    rng = random.Random(seed)
    reqs = []
    for i in range(count):
        kind = "ml" if rng.random() < ml_frac else "ip"
        n = rng.randint(lo, hi)
        seeds = [0x5E7E0000 + 2 * i + seed * 7919, 0x5E7E0000 + 2 * i + 1 + seed * 7919]
        reqs.append((kind, n, seeds))
    return reqs


def solo(E, kind, n, seeds, field, i):
    tabs = [E.gen_uniform(seeds[t], 1 << n) for t in range(2 if kind == "ip" else 1)]
    p = E.InnerProductProver(tabs[0], tabs[1], field=field) if kind == "ip" else E.MultilinearProver(tabs[0], field=field)
    return p.prove(n, E.Transcript.keccak(field, label(i)))


def same(a, b):
    return (np.array_equal(np.asarray(a.round_polys), np.asarray(b.round_polys))
            and np.array_equal(np.asarray(a.challenges), np.asarray(b.challenges))
            and np.array_equal(np.asarray(a.final_value), np.asarray(b.final_value)))


@pytest.mark.parametrize("field", [1, 3])
def test_mix_equals_alone(E, field):
    """Forty requests (IP and ML, num_vars 1..14) submitted at once with four
    slots: every proof equals the request proved alone by the single-instance
    path and, through the server, alone."""
    reqs = workload(1 + field, 40, 1, 14)
    srv = E.Server(hbm_budget=1 << 34, max_active=4)
    ids = {}
    for i, (kind, n, seeds) in enumerate(reqs):
        ids[srv.submit(E.IP if kind == "ip" else E.ML, n, E.Transcript.keccak(field, label(i)), seeds=seeds,
                       field=field)] = i
    mixed = srv.drain()
    assert len(mixed) == len(reqs)
    for rid, (proof, q, lat) in mixed.items():
        i = ids[rid]
        kind, n, seeds = reqs[i]
        assert lat >= q >= 0
        assert same(proof, solo(E, kind, n, seeds, field, i)), i
    # each request alone through a fresh server
    for i in range(0, len(reqs), 7):
        kind, n, seeds = reqs[i]
        one = E.Server(hbm_budget=1 << 34, max_active=4)
        rid = one.submit(E.IP if kind == "ip" else E.ML, n, E.Transcript.keccak(field, label(i)), seeds=seeds,
                         field=field)
        alone = one.drain()[rid][0]
        mixed_proof = [p for r, (p, _, _) in mixed.items() if ids[r] == i][0]
        assert same(alone, mixed_proof), i


def test_mix_matches_oracle(E):
    reqs = workload(11, 12, 2, 12)
    srv = E.Server(hbm_budget=1 << 34, max_active=5)
    ids = {}
    for i, (kind, n, seeds) in enumerate(reqs):
        ids[srv.submit(E.IP if kind == "ip" else E.ML, n, E.Transcript.keccak(3, label(i)), seeds=seeds)] = i
    out = srv.drain()
    for rid, (proof, _, _) in out.items():
        kind, n, seeds = reqs[ids[rid]]
        tabs = [O.gen_table(seeds[t], 1 << n) for t in range(2 if kind == "ip" else 1)]
        rp, ch, fv = O.sumcheck(O.Prover(O.IP if kind == "ip" else O.ML, O.MSB, 3, tabs), n,
                                O.Transcript(3, label=label(ids[rid])))
        assert np.array_equal(proof.round_polys, rp)
        assert np.array_equal(proof.challenges, ch)
        assert np.array_equal(proof.final_value, fv)


def test_host_tables_and_budget(E):
    """Host-table requests under a budget that admits one 2^14 IP request at
    a time: later requests wait in the queue, proofs unchanged."""
    rng = np.random.default_rng(5)
    n = 14
    per = 2 * ((1 << n) + 3 * (1 << (n - 1))) * 8 + 4096
    srv = E.Server(hbm_budget=per + per // 2, max_active=8)
    tabs = [[rng.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(2)] for _ in range(4)]
    ids = [srv.submit(E.IP, n, E.Transcript.keccak(3, label(i)), tables=tabs[i]) for i in range(4)]
    out = srv.drain()
    waits = [out[r][1] for r in ids]
    assert max(waits) > 0
    for i, r in enumerate(ids):
        ref = E.InnerProductProver(tabs[i][0], tabs[i][1]).prove(n, E.Transcript.keccak(3, label(i)))
        assert same(out[r][0], ref)


def test_rejects(E):
    srv = E.Server(hbm_budget=1 << 20, max_active=2)
    with pytest.raises(E.EffscError):     # larger than the whole budget
        srv.submit(E.IP, 20, E.Transcript.keccak(3, b"x"), seeds=[1, 2])
    with pytest.raises(E.EffscError):
        srv.submit(E.COEF, 4, E.Transcript.keccak(3, b"x"), seeds=[1])
    with pytest.raises(E.EffscError):     # transcript field differs
        srv.submit(E.IP, 4, E.Transcript.keccak(1, b"x"), seeds=[1, 2], field=3)


def test_trace_poisson(E):
    """Open-loop Poisson arrivals: latencies are measured per request and the
    proofs equal the solo proofs."""
    reqs = workload(21, 60, 4, 13)
    rng = np.random.default_rng(0)
    arrivals = np.cumsum(rng.exponential(2e-4, size=len(reqs)))
    srv = E.Server(hbm_budget=1 << 33, max_active=16)
    kinds = [E.IP if k == "ip" else E.ML for k, _, _ in reqs]
    lat, makespan, proofs = srv.run_trace(kinds, [n for _, n, _ in reqs], [s for _, _, s in reqs],
                                          [E.Transcript.keccak(3, label(i)) for i in range(len(reqs))], arrivals)
    assert (lat > 0).all() and makespan >= arrivals[-1]
    for i, (kind, n, seeds) in enumerate(reqs):
        assert same(proofs[i], solo(E, kind, n, seeds, 3, i)), i


def test_trace_host_tables(E):
    """The same trace with every request's tables in host memory (uploaded on
    admission): the proofs equal the solo proofs."""
    reqs = workload(33, 40, 4, 14)
    rng = np.random.default_rng(1)
    arrivals = np.cumsum(rng.exponential(2e-4, size=len(reqs)))
    host = [[np.asarray(E.gen_uniform(s[t], 1 << n)) for t in range(2 if k == "ip" else 1)] for k, n, s in reqs]
    srv = E.Server(hbm_budget=1 << 33, max_active=12)
    kinds = [E.IP if k == "ip" else E.ML for k, _, _ in reqs]
    lat, makespan, proofs = srv.run_trace(kinds, [n for _, n, _ in reqs], None,
                                          [E.Transcript.keccak(3, label(i)) for i in range(len(reqs))], arrivals,
                                          host_tables=host)
    assert (lat > 0).all() and makespan >= arrivals[-1]
    for i, (kind, n, seeds) in enumerate(reqs):
        assert same(proofs[i], solo(E, kind, n, seeds, 3, i)), i


def test_two_lanes_mix(E):
    """Requests of 2^22 entries and more go to the second lane (own stream,
    queue and steps); a mix of both lanes, with small requests finishing in
    tail launches, gives every request the proof it gets alone."""
    rng = random.Random(77)
    reqs = []
    for i in range(18):
        big = i % 6 == 0
        n = rng.randint(22, 23) if big else rng.randint(2, 16)
        kind = "ml" if rng.random() < 0.3 else "ip"
        reqs.append((kind, n, [0x7A7E0000 + 2 * i, 0x7A7E0001 + 2 * i]))
    srv = E.Server(hbm_budget=1 << 36, max_active=6)
    ids = {}
    for i, (kind, n, seeds) in enumerate(reqs):
        ids[srv.submit(E.IP if kind == "ip" else E.ML, n, E.Transcript.keccak(3, label(i)), seeds=seeds)] = i
    out = srv.drain()
    assert len(out) == len(reqs)
    for rid, (proof, q, lat) in out.items():
        i = ids[rid]
        kind, n, seeds = reqs[i]
        assert same(proof, solo(E, kind, n, seeds, 3, i)), i
