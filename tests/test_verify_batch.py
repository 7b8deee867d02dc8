"""Device batch verifier (effsc_verify_batch): sumcheck_verify
(src/verifier.rs:61-139) for many proofs at once, one warp per proof.

Every proof's challenges and final claim must equal the host verifier's and
the oracle's on the same inputs -- random round polynomials of degree 0..3,
both fields, with and without a hook, ragged round counts (zero included) --
and proofs made by the provers must verify (final claim == final value) while
a proof with one changed wire value must not."""
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


def to3(a, field):
    a = np.asarray(a, dtype=np.uint64).reshape(-1, field)
    out = np.zeros((a.shape[0], 3), dtype=np.uint64)
    out[:, :field] = a
    return out


@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("degree", [0, 1, 2, 3])
@pytest.mark.parametrize("hook", [b"", bytes(range(40))])
def test_random_polys_match_host_and_oracle(E, field, degree, hook):
    rng = random.Random(100 * degree + 10 * field + len(hook))
    nw = max(degree, 1)
    n = 37
    rounds = [rng.choice([0, 1, 2, 5, 13, 20]) for _ in range(n)]
    claims = np.array([[rng.randrange(O.P) for _ in range(field)] for _ in range(n)], dtype=np.uint64)
    polys = [np.array([rng.randrange(O.P) for _ in range(r * nw * field)], dtype=np.uint64).reshape(r, nw, field)
             for r in rounds]
    labels = [b"vb/%d" % i for i in range(n)]
    fin, chs = E.sumcheck_verify_batch(claims, degree, polys, [E.Transcript.keccak(field, l) for l in labels],
                                       hook=hook, field=field)
    for i in range(n):
        ch_h, fc_h = E.sumcheck_verify(list(claims[i]), degree, rounds[i], E.Transcript.keccak(field, labels[i]),
                                       polys[i], hook=hook)
        assert (chs[i] == ch_h.reshape(-1, field)).all(), i
        assert (fin[i] == fc_h).all(), i
        if field == 3:
            ch_o, fc_o = O.verify(list(claims[i]), degree, rounds[i], O.Transcript(3, label=labels[i]),
                                  polys[i], hook=hook)
            assert (chs[i] == ch_o).all() and (fin[i] == fc_o).all(), i


def test_prover_proofs_verify_and_tamper_fails(E):
    rng = np.random.default_rng(3)
    n_proofs, v = 24, 10
    claims, polys, finals, labels = [], [], [], []
    for i in range(n_proofs):
        a = rng.integers(0, O.P, size=1 << v, dtype=np.uint64)
        b = rng.integers(0, O.P, size=1 << v, dtype=np.uint64)
        s = sum(int(x) * int(y) for x, y in zip(a, b)) % O.P
        labels.append(b"vb-ip/%d" % i)
        proof = E.InnerProductProver(a, b).prove(v, E.Transcript.keccak(3, labels[-1]))
        claims.append([s, 0, 0])
        polys.append(np.asarray(proof.round_polys))
        finals.append(np.asarray(proof.final_value))
    fin, chs = E.sumcheck_verify_batch(claims, 2, polys, [E.Transcript.keccak(3, l) for l in labels])
    for i in range(n_proofs):
        assert (fin[i] == finals[i]).all(), i
    bad = [p.copy() for p in polys]
    bad[5][3, 1, 0] = (int(bad[5][3, 1, 0]) + 1) % O.P
    fin2, _ = E.sumcheck_verify_batch(claims, 2, bad, [E.Transcript.keccak(3, l) for l in labels])
    ok = [(fin2[i] == finals[i]).all() for i in range(n_proofs)]
    assert not ok[5] and sum(ok) == n_proofs - 1


def test_coefficient_degree3_proofs_verify(E):
    rng = np.random.default_rng(4)
    v = 8
    claims, polys, finals, labels = [], [], [], []
    for i in range(6):
        tabs = [rng.integers(0, O.P, size=1 << v, dtype=np.uint64) for _ in range(3)]
        s = 0
        for j in range(1 << v):
            s = (s + int(tabs[0][j]) * int(tabs[1][j]) % O.P * int(tabs[2][j])) % O.P
        labels.append(b"vb-c3/%d" % i)
        proof = E.CoefficientProver(tabs).prove(v, E.Transcript.keccak(3, labels[-1]))
        claims.append([s, 0, 0])
        polys.append(np.asarray(proof.round_polys))
        finals.append(np.asarray(proof.final_value))
    fin, _ = E.sumcheck_verify_batch(claims, 3, polys, [E.Transcript.keccak(3, l) for l in labels])
    for i in range(len(labels)):
        assert (fin[i] == finals[i]).all(), i


def test_rejects(E):
    with pytest.raises(E.EffscError):
        E.sumcheck_verify_batch([[1, 0, 0]], 4, [np.zeros((1, 4, 3), np.uint64)], [E.Transcript.keccak(3, b"x")])
    with pytest.raises(E.EffscError):     # transcript field differs
        E.sumcheck_verify_batch([[1, 0, 0]], 2, [np.zeros((1, 2, 3), np.uint64)], [E.Transcript.keccak(1, b"x")])
