"""The TMA-staged round kernel (tables of at least 2^17 entries, both
orders): proofs and post-state tables at sizes where it runs, against the
oracle, with Fp and Fp3 challenges, with the two-pass start on (Fp3 tables
into the kernel) and off (base tables into the kernel, Fp3 out), full and
partial runs."""
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


def tables(n, seed):
    g = np.random.default_rng(seed)
    return [g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(2)]


@pytest.mark.parametrize("order", ["msb", "lsb"])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("first_rounds", [True, False])
def test_full_proof_n20(E, order, field, first_rounds):
    n = 20
    a, b = tables(n, 7 + field + 2 * first_rounds + (order == "lsb"))
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p = cls(a, b, field=field)
    p.set_first_rounds(first_rounds)
    pf = p.prove(n, E.Transcript.keccak(field, b"tma"))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, field, [a, b]), n,
                            O.Transcript(field, label=b"tma"))
    assert np.array_equal(np.asarray(pf.round_polys).reshape(n, 2, field), rp[:, :, :field])
    assert np.array_equal(np.asarray(pf.challenges).reshape(n, field), ch[:, :field])
    assert np.array_equal(np.asarray(pf.final_value).reshape(field), fv[:field])


@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_partial_post_state_n19(E, order):
    """Four rounds of a 2^19 proof (the TMA kernel folds 2^17-entry tables
    in round 3 with the two-pass start off) leave the oracle's tables."""
    n, rounds = 19, 4
    a, b = tables(n, 31 + (order == "lsb"))
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p = cls(a, b)
    p.set_first_rounds(False)
    pf = p.prove(rounds, E.Transcript.keccak(3, b"tma-part"))
    orc = O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b])
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(3, label=b"tma-part"))
    assert np.array_equal(pf.round_polys, rp) and np.array_equal(pf.challenges, ch)
    for t in range(2):
        got = np.asarray(p.table(t)).reshape(-1, 3)
        assert np.array_equal(got, orc.table(t)), t
