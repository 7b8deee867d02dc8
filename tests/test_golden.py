"""Golden proofs (tests/golden/golden.json, made by tests/golden/make_golden.py).

The CPU test checks the oracle still reproduces every frozen proof; the GPU
test runs every case through the GPU provers (per-round C ABI and the
device-resident protocol) and requires the same words."""
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import table  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]


def words(a):
    return [format(int(x), "016x") for x in np.asarray(a, dtype=np.uint64).reshape(-1)]


def inputs(c):
    if c["kind"] == O.EQF:
        return table(c["seed"], 0, c["v"], c["field"] == 3), table(c["seed"], 1, 1 << c["v"], False)
    return [table(c["seed"], t, c["n"], c["field"] == 3 and c["ext_first"] and t == 0) for t in range(c["ntab"])]


def pad3(a, field):
    a = np.asarray(a, dtype=np.uint64)
    if field == 3:
        return a
    z = np.zeros(a.shape[:-1] + (3,), dtype=np.uint64)
    z[..., 0] = a[..., 0]
    return z


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_oracle_reproduces_golden(case):
    f = case["field"]
    tr = O.Transcript(f, label=case["label"].encode())
    if case["kind"] == O.EQF:
        w, p = inputs(case)
        pr = O.Prover.eq_factored(f, w, p)
    else:
        pr = O.Prover(case["kind"], case["order"], f, inputs(case))
    rp, ch, fv = O.sumcheck(pr, case["rounds"], tr, hook=bytes.fromhex(case["hook"]))
    assert words(rp) == case["round_polys"]
    assert words(ch) == case["challenges"]
    assert words(fv) == case["final_value"]


@pytest.mark.gpu
@pytest.mark.parametrize("device_path", [False, True])
@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_gpu_reproduces_golden(case, device_path):
    sys.path.insert(0, os.path.join(ROOT, "efficient-sumcheck_gb300"))
    import effsc_gpu as E
    f = case["field"]
    hook = bytes.fromhex(case["hook"])
    label = case["label"].encode()
    if case["kind"] == O.EQF:
        w, p = inputs(case)
        g = E.EqFactoredProver(w, p, field=f)
    else:
        tabs = inputs(case)
        cls = {O.ML: E.MultilinearProver, O.IP: E.InnerProductProver, O.COEF: E.CoefficientProver}[case["kind"]]
        if case["order"] == O.LSB:
            cls = {O.ML: E.MultilinearProverLSB, O.IP: E.InnerProductProverLSB,
                   O.COEF: E.CoefficientProverLSB}[case["kind"]]
        if case["kind"] == O.COEF:
            g = cls(tabs, field=f)
        else:
            g = cls(*tabs, field=f)
    t = E.Transcript.keccak(f, label)
    if device_path:
        proof = g.prove(case["rounds"], t, hook=hook)
    else:
        proof = E.sumcheck(g, case["rounds"], t, hook=(lambda r, tt: tt.absorb(hook)) if hook else None)
    assert words(pad3(proof.round_polys, f)) == case["round_polys"]
    assert words(pad3(proof.challenges, f)) == case["challenges"]
    assert words(pad3(proof.final_value, f)) == case["final_value"]
