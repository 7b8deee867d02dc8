"""The cluster tail (tables of up to 16 times one block's capacity held in the
distributed shared memory of a thread-block cluster, then handed to one CTA;
Multilinear proofs): proofs, hooks and post-state tables against the oracle
at sizes where it runs, over Fp and Fp3, and the same proof with the tail
kernels switched off.  InnerProduct proofs of the same sizes (multi-block
rounds there, then the one-block tail) are checked alongside."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    O.set_threads(os.cpu_count() or 1)
    return effsc_gpu


def tables(n, k, seed):
    g = np.random.default_rng(seed)
    return [g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(k)]


def proof_eq(pf, rp, ch, fv, n, field, d):
    return (np.array_equal(np.asarray(pf.round_polys).reshape(n, d, field), rp[:, :d, :field])
            and np.array_equal(np.asarray(pf.challenges).reshape(n, field), ch[:, :field])
            and np.array_equal(np.asarray(pf.final_value).reshape(field), fv[:field]))


@pytest.mark.parametrize("kind,field,n", [("ml", 1, 16), ("ml", 1, 18), ("ml", 1, 20), ("ml", 3, 17),
                                          ("ip", 3, 14), ("ip", 3, 16), ("ip", 3, 18), ("ip", 1, 16)])
@pytest.mark.parametrize("hook", [b"", bytes(range(32)), b"\x01\x02\x03"])
def test_full_proofs(E, kind, field, n, hook):
    k = 2 if kind == "ip" else 1
    tabs = tables(n, k, n * 10 + field + len(hook))
    cls = E.InnerProductProver if kind == "ip" else E.MultilinearProver
    p = cls(*tabs, field=field)
    label = b"cluster/%s" % kind.encode()
    pf = p.prove(n, E.Transcript.keccak(field, label), hook=hook)
    rp, ch, fv = O.sumcheck(O.Prover(O.IP if kind == "ip" else O.ML, O.MSB, field, tabs), n,
                            O.Transcript(field, label=label), hook=hook)
    assert proof_eq(pf, rp, ch, fv, n, field, k)
    q = cls(*tabs, field=field)
    q.set_tail(0)                       # one kernel per round
    pq = q.prove(n, E.Transcript.keccak(field, label), hook=hook)
    assert np.array_equal(pf.round_polys, pq.round_polys) and np.array_equal(pf.final_value, pq.final_value)


@pytest.mark.parametrize("kind,field,n,rounds", [("ml", 1, 18, 10), ("ml", 1, 18, 6), ("ip", 3, 16, 8),
                                                 ("ip", 3, 16, 5), ("ip", 1, 16, 9)])
def test_partial_post_state(E, kind, field, n, rounds):
    """A partial run whose last rounds ran in the cluster tail leaves the
    oracle's tables (the runner's finalize included)."""
    k = 2 if kind == "ip" else 1
    tabs = tables(n, k, 99 + n + rounds)
    cls = E.InnerProductProver if kind == "ip" else E.MultilinearProver
    p = cls(*tabs, field=field)
    pf = p.prove(rounds, E.Transcript.keccak(field, b"cl-part"))
    orc = O.Prover(O.IP if kind == "ip" else O.ML, O.MSB, field, tabs)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"cl-part"))
    assert np.array_equal(np.asarray(pf.round_polys).reshape(rounds, k, field), rp[:, :k, :field])
    for t in range(k):
        got = np.asarray(p.table(t)).reshape(-1, field)
        assert np.array_equal(got, orc.table(t)[:, :field]), t


def test_cluster_tail_runs(E):
    """The cluster kernel is the one that runs for an ML proof of 2^18 entries
    (one launch for the last rounds)."""
    v = tables(18, 1, 5)[0]
    p = E.MultilinearProver(v, field=1)
    E.launch_count_reset()
    p.prove(18, E.Transcript.keccak(1, b"cl"), use_graph=False)
    launches = E.launch_count()
    q = E.MultilinearProver(v, field=1)
    q.set_tail(0)
    E.launch_count_reset()
    q.prove(18, E.Transcript.keccak(1, b"cl"), use_graph=False)
    assert launches < E.launch_count() // 2
