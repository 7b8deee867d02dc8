"""GPU parity: every prover, order and field, through the C ABI, against the
oracle on the same seeded inputs and transcript.  Bit-exact (integer work)."""
import os
import random
import sys
import zlib

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def E():
    sys.path.insert(0, os.path.join(ROOT, "efficient-sumcheck_gb300"))
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def to3(a, field):
    """Pad the trailing component axis of GPU output (field words) to 3."""
    a = np.asarray(a, dtype=np.uint64)
    if field == 3:
        return a
    z = np.zeros(a.shape[:-1] + (3,), dtype=np.uint64)
    z[..., 0] = a[..., 0]
    return z


def tab3(g, i, field):
    return to3(g.table(i).reshape(-1, field), field)


def rand_table(rng, n, ext):
    g = np.random.default_rng(rng.randrange(1 << 62))
    if ext:
        return g.integers(0, O.P, size=(n, 3), dtype=np.uint64)
    return g.integers(0, O.P, size=n, dtype=np.uint64)


KINDS = {
    "ml": (O.ML, 1), "ip": (O.IP, 2), "c1": (O.COEF, 1), "c2": (O.COEF, 2), "c3": (O.COEF, 3),
}


def gpu_prover(E, kind, order, field, tabs, repr=0):
    k = {"ml": "Multilinear", "ip": "InnerProduct", "c1": "Coefficient", "c2": "Coefficient", "c3": "Coefficient"}[kind]
    cls = getattr(E, k + "Prover" + ("LSB" if order == O.LSB else ""))
    if kind == "ml":
        return cls(tabs[0], field=field, repr=repr)
    if kind == "ip":
        return cls(tabs[0], tabs[1], field=field, repr=repr)
    return cls(tabs, field=field, repr=repr)


def n_rounds(n):
    return max(1, (n - 1).bit_length()) if n > 1 else 1


def check_proof(proof, field, rp, ch, fv):
    assert (to3(proof.round_polys, field) == rp).all(), "round polynomials differ"
    assert (to3(proof.challenges, field) == ch).all(), "challenges differ"
    assert (to3(proof.final_value, field) == fv).all(), "final value differs"


SIZES = [1, 2, 3, 4, 5, 8, 13, 16, 33, 64, 100, 1024, 4099, 1 << 14, (1 << 16) + 3]


@pytest.mark.parametrize("kind", ["ml", "ip", "c1", "c2", "c3"])
@pytest.mark.parametrize("order", [O.MSB, O.LSB])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("n", SIZES)
def test_host_runner_matches_oracle(E, kind, order, field, n):
    okind, ntab = KINDS[kind]
    if kind == "ip" and order == O.LSB and n % 2 and n > 1:
        pytest.skip("covered by test_ip_lsb_odd_round0_panics")
    rng = random.Random(zlib.crc32(repr((kind, order, field, n)).encode()))
    # c3 keeps the eq * f * g shape: first table Fp3, the others base
    tabs = [rand_table(rng, n, field == 3 and kind == "c3" and i == 0) for i in range(ntab)]
    rounds = n_rounds(n) + (1 if n < 64 else 0)
    label = b"effsc-gpu/test"
    orc = O.Prover(okind, order, field, tabs)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=label))
    g = gpu_prover(E, kind, order, field, tabs)
    proof = E.sumcheck(g, rounds, E.Transcript.keccak(field, label))
    check_proof(proof, field, rp, ch, fv)
    for i in range(ntab):
        assert (tab3(g, i, field) == orc.table(i)).all(), "post-state table %d differs" % i


@pytest.mark.parametrize("kind", ["ml", "ip", "c3"])
@pytest.mark.parametrize("order", [O.MSB, O.LSB])
@pytest.mark.parametrize("n", [16, 1 << 12, (1 << 18)])
@pytest.mark.parametrize("use_graph", [False, True])
def test_device_path_matches_oracle(E, kind, order, n, use_graph):
    okind, ntab = KINDS[kind]
    field = 3
    rng = random.Random(n + 7 * order)
    tabs = [rand_table(rng, n, kind == "c3" and i == 0) for i in range(ntab)]
    rounds = n_rounds(n)
    hook = bytes(range(32))
    orc = O.Prover(okind, order, field, tabs)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"dev"), hook=hook)
    g = gpu_prover(E, kind, order, field, tabs)
    t = E.Transcript.keccak(field, b"dev")
    proof = g.prove(rounds, t, hook=hook, use_graph=use_graph)
    check_proof(proof, field, rp, ch, fv)
    # the transcript continues identically on the host afterwards
    to = O.Transcript(field, label=b"dev")
    O.sumcheck(O.Prover(okind, order, field, tabs), rounds, to, hook=hook)
    assert [int(x) for x in t.challenge()] == [int(x) for x in to.challenge()]
    # reset + replay (cached graph) gives the same proof
    g.reset()
    proof2 = g.prove(rounds, E.Transcript.keccak(field, b"dev"), hook=hook, use_graph=use_graph)
    check_proof(proof2, field, rp, ch, fv)


@pytest.mark.parametrize("v", [0, 1, 2, 3, 4, 5, 8, 13, 16, 17, 19])
@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("device_path", [False, True])
def test_eq_factored_matches_oracle(E, v, field, device_path):
    rng = random.Random(1000 + v)
    w = rand_table(rng, v, field == 3) if v else np.zeros((0, 3) if field == 3 else (0,), np.uint64)
    plen = max(1, (1 << v) - (1 if v > 2 else 0))
    p = rand_table(rng, plen, False)
    rounds = max(v, 1)
    w3 = O.as_table(w) if v else np.zeros((0, 3), np.uint64)
    orc = O.Prover.eq_factored(field, w3, p)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(field, label=b"eqf"), hook=b"hk")
    g = E.EqFactoredProver(w, p, field=field)
    if device_path:
        proof = g.prove(rounds, E.Transcript.keccak(field, b"eqf"), hook=b"hk")
    else:
        proof = E.sumcheck(g, rounds, E.Transcript.keccak(field, b"eqf"), hook=lambda r, t: t.absorb(b"hk"))
    check_proof(proof, field, rp, ch, fv)
    for i in range(3):
        assert (tab3(g, i, field) == orc.table(i)).all()


def test_eq_factored_partial_16_of_24_shape(E):
    # config-3 shape scaled down: v = 12, 8 partial rounds, 32-byte hook
    rng = random.Random(3)
    v, rounds = 12, 8
    w = rand_table(rng, v, True)
    f = rand_table(rng, 1 << v, False)
    g_ = rand_table(rng, 1 << v, False)
    p = np.array([int(a) * int(b) % O.P for a, b in zip(f, g_)], dtype=np.uint64)
    hook = bytes(range(32))
    orc = O.Prover.eq_factored(3, w, p)
    rp, ch, fv = O.sumcheck(orc, rounds, O.Transcript(3, label=b"c3"), hook=hook)
    gp = E.EqFactoredProver(w, p)
    proof = gp.prove(rounds, E.Transcript.keccak(3, b"c3"), hook=hook)
    check_proof(proof, 3, rp, ch, fv)
    # the coefficient prover on [eq(w, .), f, g] proves the same sum
    eq = O.build_eq_table(w)
    assert (E.build_eq_table(w) == eq).all()
    oc = O.Prover(O.COEF, O.MSB, 3, [eq, f, g_])
    rp3, ch3, fv3 = O.sumcheck(oc, rounds, O.Transcript(3, label=b"c3"), hook=hook)
    gc = E.CoefficientProver([eq, f, g_])
    proof3 = gc.prove(rounds, E.Transcript.keccak(3, b"c3"), hook=hook)
    check_proof(proof3, 3, rp3, ch3, fv3)


def test_ip_lsb_odd_round0_panics(E):
    a = np.arange(1, 6, dtype=np.uint64)
    g = E.InnerProductProverLSB(a, a)
    with pytest.raises(E.ReferencePanic):
        g.round(None)


def test_unequal_lengths_panic(E):
    with pytest.raises(E.ReferencePanic):
        E.InnerProductProver(np.arange(4, dtype=np.uint64), np.arange(5, dtype=np.uint64))


def test_partial_then_continue_equals_full(E):
    rng = random.Random(5)
    n, split = 1 << 10, 4
    a, b = rand_table(rng, n, False), rand_table(rng, n, False)
    full = E.InnerProductProver(a, b)
    pf = E.sumcheck(full, 10, E.Transcript.keccak(3, b"s"))
    part = E.InnerProductProver(a, b)
    t = E.Transcript.keccak(3, b"s")
    p1 = part.prove(split, t)                       # device path
    p2 = E.sumcheck(part, 10 - split, t)            # then the host runner
    assert (np.concatenate([p1.round_polys, p2.round_polys]) == pf.round_polys).all()
    assert (np.concatenate([p1.challenges, p2.challenges]) == pf.challenges).all()
    assert (p2.final_value == pf.final_value).all()


def test_test_transcript_base_challenges(E):
    # SanityTranscript semantics: Fp3 challenges are embedded base values
    rng = random.Random(6)
    n = 1 << 9
    a, b = rand_table(rng, n, False), rand_table(rng, n, False)
    orc = O.Prover(O.IP, O.MSB, 3, [a, b])
    rp, ch, fv = O.sumcheck(orc, 9, O.Transcript(3, seed=99))
    proof = E.sumcheck(E.InnerProductProver(a, b), 9, E.Transcript.test(3, 99))
    check_proof(proof, 3, rp, ch, fv)


def test_montgomery_boundary(E):
    rng = random.Random(7)
    n = 1 << 8
    a, b = rand_table(rng, n, False), rand_table(rng, n, True)
    R = (1 << 64) % O.P
    mont = lambda x: np.array([int(v) * R % O.P for v in np.asarray(x).reshape(-1)], dtype=np.uint64).reshape(np.asarray(x).shape)
    canon = lambda x: np.array([int(v) * pow(R, -1, O.P) % O.P for v in np.asarray(x).reshape(-1)], dtype=np.uint64).reshape(np.asarray(x).shape)
    g1 = E.InnerProductProver(a, b)
    p1 = E.sumcheck(g1, 8, E.Transcript.keccak(3, b"m"))
    g2 = E.InnerProductProver(mont(a), mont(b), repr=E.MONTGOMERY)
    p2 = E.sumcheck(g2, 8, E.Transcript.keccak(3, b"m", repr=E.MONTGOMERY))
    assert (canon(p2.round_polys) == p1.round_polys).all()
    assert (canon(p2.final_value) == p1.final_value).all()
    assert (canon(g2.table(0)) == g1.table(0)).all()


@pytest.mark.parametrize("n", [0, 1, 2, 5, 8, 1000, 1 << 15])
@pytest.mark.parametrize("field", [1, 3])
def test_standalone_fold(E, n, field):
    rng = random.Random(n)
    v = rand_table(rng, n, field == 3)
    w = [rng.randrange(O.P) for _ in range(field)]
    out = E.fold(v, w, field=field)
    orc = O.Prover(O.ML, O.MSB, field, [v if n else np.zeros(0, np.uint64)])
    orc.finalize(w + [0] * (3 - field))
    assert (to3(out.reshape(-1, field), field) == orc.table(0)).all()


def test_verifier_accepts_gpu_proofs(E):
    rng = random.Random(8)
    n = 1 << 12
    a, b = rand_table(rng, n, False), rand_table(rng, n, False)
    s = sum(int(x) * int(y) for x, y in zip(a, b)) % O.P
    proof = E.InnerProductProver(a, b).prove(12, E.Transcript.keccak(3, b"acc"))
    ch, fc = E.sumcheck_verify([s, 0, 0], 2, 12, E.Transcript.keccak(3, b"acc"), proof.round_polys)
    assert (ch == proof.challenges).all() and (fc == proof.final_value).all()


def test_uniform_generator_matches_oracle(E):
    for seed in (1, 0xABCDEF):
        assert (E.gen_uniform(seed, 5000) == O.gen_table(seed, 5000)).all()


def test_kernels_launch(E):
    E.launch_count_reset()
    rng = random.Random(9)
    a = rand_table(rng, 1 << 12, False)
    p = E.InnerProductProver(a, a)
    p.set_tail(0)        # one kernel per round
    p.set_persistent(0)
    p.prove(12, E.Transcript.keccak(3, b"k"), use_graph=False)
    assert E.launch_count() >= 12
    E.launch_count_reset()
    p.reset()
    p.set_persistent(1 << 21)   # rounds 3..11 in one cooperative launch
    p.prove(12, E.Transcript.keccak(3, b"k"), use_graph=False)
    assert 2 <= E.launch_count() <= 8
    E.launch_count_reset()
    p.reset()
    p.set_tail(None)     # all 12 rounds in the one-block tail kernel, the final folds, the read-back gather
    p.prove(12, E.Transcript.keccak(3, b"k"), use_graph=False)
    assert 1 <= E.launch_count() <= 4


def test_transcript_latency_probe(E):
    """effsc_diag_transcript_latency: a round step (send + challenge) costs
    at least one permutation and stays within a few microseconds."""
    import ctypes
    perm, step = ctypes.c_double(), ctypes.c_double()
    assert E.load().effsc_diag_transcript_latency(E.Context.default().h, ctypes.byref(perm), ctypes.byref(step)) == 0
    assert 0 < perm.value <= step.value < 50_000
