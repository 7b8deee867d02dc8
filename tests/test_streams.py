"""Streams (src/streams/) and tables read in place from host memory.

reorder_vec_msb and the stream claims against Python restatements; provers
over host-resident tables (pageable numpy arrays and a memory-mapped
FileStream) against the oracle, through every schedule (two-pass start, TMA
rounds, tail, per-round API)."""
import numpy as np
import pytest

import bigint_ref as R
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def brev(i, v):
    return int(format(i, "0%db" % v)[::-1], 2) if v else 0


@pytest.mark.parametrize("v", [0, 1, 2, 4, 8, 12])
@pytest.mark.parametrize("ncomp", [1, 3])
def test_reorder_vec_msb(E, v, ncomp):
    n = 1 << v
    g = np.random.default_rng(v + ncomp)
    x = g.integers(0, O.P, size=(n, 3) if ncomp == 3 else n, dtype=np.uint64)
    y = E.reorder_vec_msb(x)
    for i in range(n):
        assert np.array_equal(y[i], x[brev(i, v)])
    assert np.array_equal(E.reorder_vec_msb(y), x)          # msb_reorder_roundtrip


def test_reorder_rejects_non_power_of_two(E):
    with pytest.raises(E.ReferencePanic):
        E.reorder_vec_msb(np.arange(6, dtype=np.uint64))


@pytest.mark.parametrize("ntab", [1, 2, 3])
@pytest.mark.parametrize("ext", [False, True])
def test_claims_match_bigint(E, ntab, ext):
    g = np.random.default_rng(10 * ntab + ext)
    n = 1 << 11
    tabs = [g.integers(0, O.P, size=(n, 3) if ext else n, dtype=np.uint64) for _ in range(ntab)]
    want = R.ZERO
    for i in range(n):
        p = R.ONE
        for t in tabs:
            p = R.mul(p, tuple(int(x) for x in t[i]) if ext else R.lift(t[i]))
        want = R.add(want, p)
    got = E.multivariate_product_claim(tabs, field=3)
    assert tuple(int(x) for x in got) == want
    if ntab == 1:
        assert tuple(int(x) for x in E.multivariate_claim(E.MemoryStream(tabs[0]), field=3)) == want


@pytest.mark.parametrize("n", [8, 12, 14, 15, 17])
@pytest.mark.parametrize("tail", [None, 0])
@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_ip_over_host_tables(E, n, tail, order):
    """From 2^14 entries the two-pass start's first pass reads the host
    tables once and copies them to the device for the second."""
    g = np.random.default_rng(n)
    a = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    b = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    a0, b0 = a.copy(), b.copy()
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p = cls.from_host([a, b], field=3)
    p.set_tail(tail)
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB if order == "msb" else O.LSB, 3, [a, b]), n,
                            O.Transcript(3, label=b"host"))
    for use_graph in (True, True, False):
        p.reset()
        proof = p.prove(n, E.Transcript.keccak(3, b"host"), use_graph=use_graph)
        assert np.array_equal(proof.round_polys, rp)
        assert np.array_equal(proof.final_value, fv)
    assert np.array_equal(a, a0) and np.array_equal(b, b0)
    # the per-round API over the same host tables
    q = cls.from_host([a, b], field=3)
    proof = E.sumcheck(q, n, E.Transcript.keccak(3, b"host"))
    assert np.array_equal(proof.round_polys, rp)
    assert np.array_equal(proof.final_value, fv)


@pytest.mark.parametrize("rounds", [4, 5, 9])
@pytest.mark.parametrize("order", ["msb", "lsb"])
def test_ip_host_tables_partial_post_state(E, rounds, order):
    """Partial runs over host tables leave the tables a device-table prover
    leaves."""
    n = 15
    g = np.random.default_rng(rounds)
    a = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    b = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    cls = E.InnerProductProver if order == "msb" else E.InnerProductProverLSB
    p = cls.from_host([a, b], field=3)
    q = cls(a, b, field=3)
    x = p.prove(rounds, E.Transcript.keccak(3, b"hp"))
    y = q.prove(rounds, E.Transcript.keccak(3, b"hp"))
    assert np.array_equal(x.round_polys, y.round_polys)
    assert np.array_equal(x.final_value, y.final_value)
    for t in range(2):
        assert np.array_equal(p.table(t), q.table(t))


def test_ip_fp_field_over_host_tables_uses_plain_loads(E):
    """Fp field, no two-pass start: round 1 reads the host tables directly
    (the TMA-staged kernel is kept to device memory)."""
    n = 18
    g = np.random.default_rng(3)
    a = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    b = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    proof = E.InnerProductProver.from_host([a, b], field=1).prove(n, E.Transcript.keccak(1, b"f"))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB, 1, [a, b]), n, O.Transcript(1, label=b"f"))
    assert np.array_equal(proof.round_polys.reshape(n, 2), rp[:, :, 0])
    assert np.array_equal(proof.final_value.reshape(1), fv[:1])


def test_multilinear_from_file_stream(E, tmp_path):
    n = 14
    g = np.random.default_rng(7)
    v = g.integers(0, O.P, size=1 << n, dtype=np.uint64)
    path = str(tmp_path / "evals.bin")
    E.FileStream.write_to_file(path, v)
    fs = E.FileStream(path)
    assert fs.num_variables() == n and int(fs.evaluation(5)) == int(v[5])
    ml = E.MultilinearProver.from_host([fs.evaluations], field=3)
    proof = ml.prove(n, E.Transcript.keccak(3, b"file"))
    rp, ch, fv = O.sumcheck(O.Prover(O.ML, O.MSB, 3, [v]), n, O.Transcript(3, label=b"file"))
    assert np.array_equal(proof.round_polys, rp)
    assert np.array_equal(proof.final_value, fv)
    # the claim of the stream is the sum the proof starts from: h(0) + h(1) of round 0
    total = 0
    for x in v:
        total = (total + int(x)) % O.P
    assert tuple(int(x) for x in E.multivariate_claim(fs, field=3)) == (total, 0, 0)
    del ml
    E.FileStream.delete_file(path)


@pytest.mark.parametrize("n", [15, 17])
@pytest.mark.parametrize("rounds", [None, 5])
def test_ip_pinned_host_tables_chunked_upload(E, n, rounds):
    """Pinned host tables (MSB): uploaded in chunks on a copy stream while the
    first pass runs over the chunks already on the device; proofs and the
    tables after partial runs equal a device-table prover's and the oracle's,
    with and without a graph."""
    torch = pytest.importorskip("torch")
    g = np.random.default_rng(100 + n)
    src = [g.integers(0, O.P, size=1 << n, dtype=np.uint64) for _ in range(2)]
    pinned = [torch.empty(1 << n, dtype=torch.int64, pin_memory=True) for _ in range(2)]
    views = [t.numpy().view(np.uint64) for t in pinned]
    for v, x in zip(views, src):
        v[:] = x
    nr = n if rounds is None else rounds
    p = E.InnerProductProver.from_host(views, field=3)
    q = E.InnerProductProver(src[0], src[1], field=3)
    y = q.prove(nr, E.Transcript.keccak(3, b"pin"))
    for use_graph in (False, True, True):
        p.reset()
        x = p.prove(nr, E.Transcript.keccak(3, b"pin"), use_graph=use_graph)
        assert np.array_equal(x.round_polys, y.round_polys)
        assert np.array_equal(x.challenges, y.challenges)
        assert np.array_equal(x.final_value, y.final_value)
    if rounds is not None:
        for t in range(2):
            assert np.array_equal(p.table(t), q.table(t))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB, 3, src), nr, O.Transcript(3, label=b"pin"))
    assert np.array_equal(x.round_polys, rp)
    assert np.array_equal(x.final_value, fv)
    for v, x0 in zip(views, src):
        assert np.array_equal(v, x0)
