"""The crate's public algebra helpers and legacy runners (src/lib.rs:51-57)
on the GPU, against the oracle:

- compute_sumcheck_polynomial (src/multilinear_sumcheck.rs:86-124) and
  fused_fold_and_compute_polynomial (:189-254), power-of-two lengths (the
  fused pass) and others (the reference's fold-then-compute fallback,
  :194-196), lengths below 4, both fields; the reference's own property:
  fused == fold then compute (tests/multilinear_sumcheck.rs:253-296);
- inner_product_sumcheck[_partial] (sends (c0, c2) per round) and
  multilinear_sumcheck[_partial] (sends (s0, s1)), full and partial runs,
  power-of-two and padded lengths, with a hook, against the oracle's legacy
  runner (tests/inner_product_sumcheck.rs:298-351 restated)."""
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


def rand(rng, n, field):
    shape = (n,) if field == 1 else (n, 3)
    return np.array([rng.randrange(O.P) for _ in range(n * field)], dtype=np.uint64).reshape(shape)


def to3(x, field):
    a = np.asarray(x, dtype=np.uint64).reshape(-1, field)
    z = np.zeros((a.shape[0], 3), dtype=np.uint64)
    z[:, :field] = a
    return z


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 5, 8, 12, 64, 1000, 1 << 12])
@pytest.mark.parametrize("field", [1, 3])
def test_compute_sumcheck_polynomial(E, n, field):
    rng = random.Random(100 * n + field)
    v = rand(rng, n, field)
    s0, s1 = E.compute_sumcheck_polynomial(v, field=field)
    if n == 0:
        want = np.zeros((2, 3), np.uint64)
    else:
        # the oracle's Multilinear round 0 (legacy pair (s0, s1))
        _, aux = O.Prover(O.ML, O.MSB, field, [v]).round(None, aux=True)
        want = aux
    assert np.array_equal(to3(s0, field)[0], want[0]) and np.array_equal(to3(s1, field)[0], want[1])


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 5, 7, 8, 12, 64, 1000, 1 << 12, 1 << 15])
@pytest.mark.parametrize("field", [1, 3])
def test_fused_fold_and_compute_polynomial(E, n, field):
    rng = random.Random(7 * n + field)
    v = rand(rng, n, field)
    w = [rng.randrange(O.P) for _ in range(field)]
    folded, (s0, s1) = E.fused_fold_and_compute_polynomial(v, np.array(w, dtype=np.uint64), field=field)
    # fused == fold then compute, on the GPU and against the oracle
    f2 = E.fold(v, np.array(w, dtype=np.uint64), field=field)
    assert np.array_equal(np.asarray(folded).reshape(-1), np.asarray(f2).reshape(-1))
    c0, c1 = E.compute_sumcheck_polynomial(f2, field=field) if n else (np.zeros(field, np.uint64),) * 2
    assert np.array_equal(np.asarray(s0).reshape(-1), np.asarray(c0).reshape(-1))
    assert np.array_equal(np.asarray(s1).reshape(-1), np.asarray(c1).reshape(-1))
    if n:
        orc = O.Prover(O.ML, O.MSB, field, [v])
        orc.round(None)
        _, aux = orc.round(w + [0] * (3 - field), aux=True)
        assert np.array_equal(to3(folded, field), orc.table(0))
        assert np.array_equal(to3(s0, field)[0], aux[0]) and np.array_equal(to3(s1, field)[0], aux[1])


def legacy_oracle(kind, tabs, rounds, label, hook):
    orc = O.Prover(kind, O.MSB, 2 if kind == O.IP else 1, tabs)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(3, label=label), hook=hook, legacy=True)
    return orc, rp, ch, fv


@pytest.mark.parametrize("n", [1, 2, 5, 8, 100, 1 << 10])
@pytest.mark.parametrize("partial", [False, True])
def test_inner_product_sumcheck_legacy(E, n, partial):
    rng = random.Random(n + 1000 * partial)
    a, b = rand(rng, n, 1), rand(rng, n, 1)
    full = (n - 1).bit_length()
    rounds = max(0, full - 2) if partial else full
    hook = bytes(range(5))
    t = E.Transcript.keccak(3, b"legacy-ip")
    got = (E.inner_product_sumcheck_partial(a, b, t, rounds, hook=lambda r, tr: tr.absorb(hook)) if partial
           else E.inner_product_sumcheck(a, b, t, hook=lambda r, tr: tr.absorb(hook)))
    orc, rp, ch, fv = legacy_oracle(O.IP, [a, b], rounds, b"legacy-ip", hook)
    msgs = np.array([[m[0], m[1]] for m in got.prover_messages], dtype=np.uint64).reshape(rounds, 2, 3)
    assert np.array_equal(msgs, rp)
    assert np.array_equal(np.array(got.verifier_messages, dtype=np.uint64).reshape(rounds, 3), ch)
    assert np.array_equal(got.a, orc.table(0)) and np.array_equal(got.b, orc.table(1))
    if orc.table(0).shape[0] == 1:
        assert np.array_equal(got.final_evaluations[0], orc.table(0)[0])
        assert np.array_equal(got.final_evaluations[1], orc.table(1)[0])


@pytest.mark.parametrize("n", [1, 2, 5, 8, 100, 1 << 10])
@pytest.mark.parametrize("partial", [False, True])
def test_multilinear_sumcheck_legacy(E, n, partial):
    rng = random.Random(n + 2000 * partial)
    v = rand(rng, n, 1)
    full = (n - 1).bit_length()
    rounds = max(0, full - 2) if partial else full
    hook = b"\x09\x08"
    t = E.Transcript.keccak(3, b"legacy-ml")
    got = (E.multilinear_sumcheck_partial(v, t, rounds, hook=lambda r, tr: tr.absorb(hook)) if partial
           else E.multilinear_sumcheck(v, t, hook=lambda r, tr: tr.absorb(hook)))
    orc, rp, ch, fv = legacy_oracle(O.ML, [v], rounds, b"legacy-ml", hook)
    msgs = np.array([[m[0], m[1]] for m in got.prover_messages], dtype=np.uint64).reshape(rounds, 2, 3)
    assert np.array_equal(msgs, rp)
    assert np.array_equal(np.array(got.verifier_messages, dtype=np.uint64).reshape(rounds, 3), ch)
    assert np.array_equal(got.values, orc.table(0))
    if orc.table(0).shape[0] == 1:
        assert np.array_equal(got.final_evaluation, orc.table(0)[0])


def test_legacy_round_count_panics(E):
    """num_rounds beyond log2(next_pow2(len)) panics in the reference
    (src/inner_product_sumcheck.rs:317-322, src/multilinear_sumcheck.rs:276-280)."""
    v = np.arange(5, dtype=np.uint64)
    with pytest.raises(E.ReferencePanic):
        E.inner_product_sumcheck_partial(v, v, E.Transcript.keccak(3, b"x"), 4)
    with pytest.raises(E.ReferencePanic):
        E.multilinear_sumcheck_partial(v, E.Transcript.keccak(3, b"x"), 4)
