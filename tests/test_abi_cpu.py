"""CPU tests of the C ABI: exports, and the host-side parts (transcript,
verifier, seeds) against the oracle.  No GPU call is made here."""
import os
import random
import re

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "effsc_gpu.h")


@pytest.fixture(scope="module")
def E():
    import importlib
    import sys
    sys.path.insert(0, os.path.join(ROOT, "efficient-sumcheck_gb300"))
    build = importlib.import_module("build")
    build.build()
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(effsc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(E):
    import ctypes
    lib = ctypes.CDLL(E.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), s
    from effsc_gpu._lib import SIGNATURES
    assert sorted(SIGNATURES) == syms


def test_table_seed_matches_oracle(E):
    for s, t in [(0, 0), (1, 2), (0xDEADBEEF, 7), (2**64 - 1, 3)]:
        assert E.table_seed(s, t) == O.table_seed(s, t)


@pytest.mark.parametrize("field", [1, 3])
def test_keccak_transcript_matches_oracle(E, field):
    rng = random.Random(field)
    label = b"effsc-gpu/ip/v1"
    a = E.Transcript.keccak(field, label)
    b = O.Transcript(field, label=label)
    for step in range(40):
        op = rng.randrange(4)
        if op == 0:
            v = [rng.randrange(O.P) for _ in range(field)]
            a.send(v)
            b.send(v + [0] * (3 - field))
        elif op == 1:
            data = bytes(rng.randrange(256) for _ in range(rng.randrange(0, 300)))
            a.absorb(data)
            b.absorb(data)
        elif op == 2:
            n = rng.randrange(1, 200)
            assert a.squeeze(n) == b.squeeze(n)
        else:
            ca, cb = a.challenge(), b.challenge()
            assert [int(x) for x in ca] == [int(x) for x in cb[:field]]


@pytest.mark.parametrize("field", [1, 3])
def test_test_transcript_matches_oracle(E, field):
    a = E.Transcript.test(field, 99)
    b = O.Transcript(field, seed=99)
    for _ in range(20):
        a.send([5] * field)
        assert [int(x) for x in a.challenge()] == [int(x) for x in b.challenge()[:field]]


def test_transcript_montgomery_repr(E):
    a = E.Transcript.keccak(3, b"m", repr=E.MONTGOMERY)
    b = E.Transcript.keccak(3, b"m")
    v = [11, 22, 33]
    a.send([x * (2**64) % O.P for x in v])
    b.send(v)
    ca, cb = a.challenge(), b.challenge()
    R_INV = pow(2**64, -1, O.P)
    assert [int(x) * R_INV % O.P for x in ca] == [int(x) for x in cb]


@pytest.mark.parametrize("deg_kind", [(1, O.ML, 1), (2, O.IP, 2), (3, O.COEF, 3)])
def test_verifier_matches_oracle(E, deg_kind):
    degree, kind, ntab = deg_kind
    rng = random.Random(degree)
    v = 6
    tabs = [np.array([rng.randrange(O.P) for _ in range(1 << v)], dtype=np.uint64) for _ in range(ntab)]
    pr = O.Prover(kind, O.MSB, 3, tabs)
    hook = bytes(range(32))
    rp, ch, fv = O.sumcheck(pr, v, O.Transcript(3, label=b"v"), hook=hook)
    s = 0
    for i in range(1 << v):
        p = 1
        for t in tabs:
            p = p * int(t[i]) % O.P
        s = (s + p) % O.P
    ch_g, fc_g = E.sumcheck_verify([s, 0, 0], degree, v, E.Transcript.keccak(3, b"v"), rp, hook=hook)
    ch_o, fc_o = O.verify([s, 0, 0], degree, v, O.Transcript(3, label=b"v"), rp, hook=hook)
    assert (ch_g == ch_o).all() and (fc_g == fc_o).all() and (fc_g == fv).all()


def test_ctx_create_without_gpu_fails_cleanly(E):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(E.EffscError):
        E.Context(0)
