"""Multiplication by the Fp3 non-residue W (csrc/gl_w.h, used by every
kernel that prepares an Fp3 multiplier) against Python integers: edge
operands (0, 1, p - 1, W, powers of two, values near the 7x carry
boundaries), non-canonical 64-bit inputs and random values.  The header is
plain C, compiled here for the host."""
import os
import random
import shutil
import subprocess

import pytest

P = 2**64 - 2**32 + 1
W = 0xFFFFFFF800000001
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "efficient-sumcheck_gb300", "csrc")

HARNESS = r"""
#include <stdio.h>
#include "gl_w.h"
int main(void) {
    unsigned long long x;
    while (scanf("%llu", &x) == 1) printf("%llu\n", (unsigned long long)gl_mul_w(x));
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("glw")
    src, exe = d / "t.c", d / "t"
    src.write_text(HARNESS)
    subprocess.check_call([cc, "-O2", "-I", CSRC, str(src), "-o", str(exe)])
    return str(exe)


def run(exe, xs):
    out = subprocess.run([exe], input="\n".join(map(str, xs)), capture_output=True, text=True, check=True).stdout
    return [int(v) for v in out.split()]


def test_edges(harness):
    xs = [0, 1, 2, 7, P - 1, P - 2, W, 2**32 - 1, 2**32, 2**33, 2**61, 2**63, (P - 1) // 2]
    xs += [(2**64 - 1) // 7 + d for d in range(-4, 5)] + [(2**61) + d for d in range(-3, 4)]
    xs = [x for x in xs if 0 <= x < P]
    assert run(harness, xs) == [(W * x) % P for x in xs]


def test_non_canonical_inputs(harness):
    xs = [P, P + 1, 2**64 - 1, 2**64 - 2**32, 2**64 - 7] + [random.Random(1).randrange(P, 2**64) for _ in range(100)]
    assert run(harness, xs) == [(W * x) % P for x in xs]


def test_random(harness):
    rng = random.Random(2026)
    xs = [rng.randrange(P) for _ in range(50000)]
    assert run(harness, xs) == [(W * x) % P for x in xs]
