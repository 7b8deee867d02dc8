"""Generate the committed golden proofs in tests/golden/golden.json.

The reference crate ships no golden vectors (its tests are property tests) and
cannot be built here, so these fixtures come from the oracle in oracle/ after
it passed the big-integer and property pins of tests/test_oracle.py.  They
freeze the exact proofs (round polynomials, challenges, final value) for small
seeded cases of every prover, order and field, with the Keccak transcript, so
any later change to the oracle or to the GPU path that alters a value fails.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")

CASES = [
    # name, kind, order, field, n, ntab, ext_first, rounds, hook
    ("ml_msb_fp_n20", O.ML, O.MSB, 1, 1 << 10, 1, False, 10, ""),
    ("ml_msb_fp_np2", O.ML, O.MSB, 1, 13, 1, False, 5, ""),
    ("ml_lsb_fp3_n9", O.ML, O.LSB, 3, 1 << 9, 1, False, 9, ""),
    ("ip_msb_fp3_n10", O.IP, O.MSB, 3, 1 << 10, 2, False, 10, ""),
    ("ip_msb_fp3_np2", O.IP, O.MSB, 3, 100, 2, False, 8, ""),
    ("ip_lsb_fp3_n10", O.IP, O.LSB, 3, 1 << 10, 2, False, 10, ""),
    ("ip_msb_fp_n8", O.IP, O.MSB, 1, 1 << 8, 2, False, 8, ""),
    ("coef3_msb_fp3_eqfg_partial", O.COEF, O.MSB, 3, 1 << 10, 3, True, 6, "000102030405060708090a0b0c0d0e0f101112131415161718191a1b1c1d1e1f"),
    ("coef3_lsb_fp3_n8", O.COEF, O.LSB, 3, 1 << 8, 3, True, 8, ""),
    ("coef2_msb_fp_n8", O.COEF, O.MSB, 1, 1 << 8, 2, False, 8, ""),
]
EQF_CASES = [
    # name, field, v, rounds, hook
    ("eqf_fp3_v10_partial", 3, 10, 6, "000102030405060708090a0b0c0d0e0f101112131415161718191a1b1c1d1e1f"),
    ("eqf_fp3_v7", 3, 7, 7, ""),
    ("eqf_fp_v6", 1, 6, 6, ""),
]


def table(seed, t, n, ext):
    if not ext:
        return O.gen_table(O.table_seed(seed, t), n)
    return np.stack([O.gen_table(O.table_seed(seed, 10 * t + c), n) for c in range(3)], axis=1)


def words(a):
    return [format(int(x), "016x") for x in np.asarray(a, dtype=np.uint64).reshape(-1)]


def main():
    out = {"note": "generated by tests/golden/make_golden.py from the oracle", "cases": []}
    for i, (name, kind, order, field, n, ntab, ext_first, rounds, hook) in enumerate(CASES):
        seed = 0xC0FFEE + i
        tabs = [table(seed, t, n, field == 3 and ext_first and t == 0) for t in range(ntab)]
        label = ("effsc-gpu/golden/" + name).encode()
        rp, ch, fv = O.sumcheck(O.Prover(kind, order, field, tabs), rounds, O.Transcript(field, label=label),
                                hook=bytes.fromhex(hook))
        out["cases"].append({"name": name, "kind": kind, "order": order, "field": field, "n": n, "ntab": ntab,
                             "ext_first": ext_first, "seed": seed, "rounds": rounds, "hook": hook,
                             "label": label.decode(), "round_polys": words(rp), "challenges": words(ch),
                             "final_value": words(fv)})
    for i, (name, field, v, rounds, hook) in enumerate(EQF_CASES):
        seed = 0xE0F00 + i
        w = table(seed, 0, v, field == 3)
        p = table(seed, 1, 1 << v, False)
        label = ("effsc-gpu/golden/" + name).encode()
        rp, ch, fv = O.sumcheck(O.Prover.eq_factored(field, w, p), rounds, O.Transcript(field, label=label),
                                hook=bytes.fromhex(hook))
        out["cases"].append({"name": name, "kind": O.EQF, "order": O.MSB, "field": field, "n": 1 << v, "v": v,
                             "seed": seed, "rounds": rounds, "hook": hook, "label": label.decode(),
                             "round_polys": words(rp), "challenges": words(ch), "final_value": words(fv)})
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", OUT, len(out["cases"]), "cases")


if __name__ == "__main__":
    main()
