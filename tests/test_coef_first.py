"""Coefficient rounds 0-2 in two passes (coef01.cuh: rounds 0 and 1 from 15
triple-product sums of one read, round 2 with the folds by r0 and r1 from a
second): proofs, challenges, final values and the tables after the run are
those of one pass per round and of the oracle, MSB and LSB, table 0 in Fp3
(an eq table) or Fp, full and partial runs, hooks, graph and direct."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def tables(E, n, seed, ext0):
    g = np.random.default_rng(seed)
    if ext0:
        w = g.integers(0, O.P, size=(n, 3), dtype=np.uint64)
        t0 = np.asarray(E.build_eq_table(w))
    else:
        t0 = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    f = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    h = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    return [t0, f, h]


def provers(E, order, tabs):
    cls = E.CoefficientProver if order == "msb" else E.CoefficientProverLSB
    p, q = cls(tabs), cls(tabs)
    q.set_first_rounds(0)
    return p, q


def same(x, y):
    assert np.array_equal(x.round_polys, y.round_polys)
    assert np.array_equal(x.challenges, y.challenges)
    assert np.array_equal(x.final_value, y.final_value)


@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("ext0", [True, False])
@pytest.mark.parametrize("n", [12, 13, 16])
def test_full_runs(E, order, ext0, n):
    tabs = tables(E, n, 10 * n + ext0 + 2 * (order == "lsb"), ext0)
    p, q = provers(E, order, tabs)
    hook = bytes(range(32))
    for use_graph in (True, True, False):
        p.reset()
        q.reset()
        x = p.prove(n, E.Transcript.keccak(3, b"c3"), hook=hook, use_graph=use_graph)
        y = q.prove(n, E.Transcript.keccak(3, b"c3"), hook=hook, use_graph=use_graph)
        same(x, y)
    rp, ch, fv = O.sumcheck(O.Prover(O.COEF, O.MSB if order == "msb" else O.LSB, 3, tabs), n,
                            O.Transcript(3, label=b"c3"), hook=hook)
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.challenges, ch)
    assert np.array_equal(x.final_value, fv)


@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("rounds", [3, 4, 7])
def test_partial_runs_post_state(E, order, rounds):
    n = 14
    tabs = tables(E, n, rounds + 50 * (order == "lsb"), True)
    p, q = provers(E, order, tabs)
    x = p.prove(rounds, E.Transcript.keccak(3, b"c3p"), hook=b"\x07")
    y = q.prove(rounds, E.Transcript.keccak(3, b"c3p"), hook=b"\x07")
    same(x, y)
    for t in range(3):
        assert np.array_equal(p.table(t), q.table(t))
    rp, ch, fv = O.sumcheck(O.Prover(O.COEF, O.MSB if order == "msb" else O.LSB, 3, tabs), rounds,
                            O.Transcript(3, label=b"c3p"), hook=b"\x07")
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.final_value, fv)


def test_bench_shape_n20(E):
    """The bench workload's shape (eq(r, .) in Fp3, f, g in Fp, 16 rounds, a
    32-byte hook) at 2^20 entries: many blocks in both passes."""
    n, rounds = 20, 16
    tabs = tables(E, n, 2026, True)
    p, q = provers(E, "msb", tabs)
    hook = bytes(range(32))
    x = p.prove(rounds, E.Transcript.keccak(3, b"c3b"), hook=hook)
    y = q.prove(rounds, E.Transcript.keccak(3, b"c3b"), hook=hook)
    same(x, y)
