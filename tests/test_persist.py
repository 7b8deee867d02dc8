"""InnerProduct rounds over Fp3 in one cooperative launch (k_persist.cu):
proofs, challenges, final values and post-state tables identical to one
launch per round and to the oracle, MSB and LSB, with and without the tail,
hooks, partial runs ending inside the persistent stretch, graph and direct
launches, base and Fp3 input tables."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def tables(n, seed, ext=False):
    g = np.random.default_rng(seed)
    shape = (1 << n, 3) if ext else (1 << n,)
    return [g.integers(0, O.P, size=shape, dtype=np.uint64) for _ in range(2)]


def pair(E, order, a, b, tail, first=2):
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p, q = cls(a, b), cls(a, b)
    for x in (p, q):
        x.set_tail(tail)
        x.set_first_rounds(first)
    p.set_persistent(1 << 21)
    q.set_persistent(0)
    return p, q


def same(x, y):
    assert np.array_equal(x.round_polys, y.round_polys)
    assert np.array_equal(x.challenges, y.challenges)
    assert np.array_equal(x.final_value, y.final_value)


@pytest.mark.parametrize("n", [5, 9, 12, 15, 18])
@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("tail", [None, 0])
def test_full_runs(E, n, order, tail):
    a, b = tables(n, 300 + n)
    p, q = pair(E, order, a, b, tail)
    hook = bytes(range(7))
    for use_graph in (True, True, False):
        p.reset()
        q.reset()
        x = p.prove(n, E.Transcript.keccak(3, b"ps"), hook=hook, use_graph=use_graph)
        y = q.prove(n, E.Transcript.keccak(3, b"ps"), hook=hook, use_graph=use_graph)
        same(x, y)
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), n,
                            O.Transcript(3, label=b"ps"), hook=hook)
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.challenges, ch)
    assert np.array_equal(x.final_value, fv)


@pytest.mark.parametrize("rounds", [2, 5, 6, 7, 9, 11])
@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_partial_runs_post_state(E, rounds, order):
    """Runs that stop inside the rounds the cooperative launch would take:
    the tables after the run (LSB: in whichever ping-pong buffer) equal the
    per-round path's and the oracle's proof prefix."""
    n = 14
    a, b = tables(n, 40 + rounds)
    p, q = pair(E, order, a, b, None)
    x = p.prove(rounds, E.Transcript.keccak(3, b"pp"))
    y = q.prove(rounds, E.Transcript.keccak(3, b"pp"))
    same(x, y)
    for t in range(2):
        assert np.array_equal(p.table(t), q.table(t))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), rounds,
                            O.Transcript(3, label=b"pp"))
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.final_value, fv)


@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("first", [0, 1, 2])
def test_ext_tables_and_first_rounds(E, order, first):
    """Fp3 input tables (the first fold leaves the caller's tables untouched
    before the cooperative rounds start) and every first-rounds level."""
    n = 13
    a, b = tables(n, 7 + first, ext=True)
    p, q = pair(E, order, a, b, None, first)
    x = p.prove(n, E.Transcript.keccak(3, b"pe"), hook=b"\x01\x02")
    y = q.prove(n, E.Transcript.keccak(3, b"pe"), hook=b"\x01\x02")
    same(x, y)
    # the caller's tables are unchanged: a second proof after reset agrees
    p.reset()
    z = p.prove(n, E.Transcript.keccak(3, b"pe"), hook=b"\x01\x02")
    same(x, z)


@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_small_limits(E, order):
    """A limit below the table sizes: the cooperative launch starts later."""
    n = 16
    a, b = tables(n, 99)
    p, q = pair(E, order, a, b, 0)
    p.set_persistent(1 << 9)
    x = p.prove(n, E.Transcript.keccak(3, b"pl"))
    y = q.prove(n, E.Transcript.keccak(3, b"pl"))
    same(x, y)
