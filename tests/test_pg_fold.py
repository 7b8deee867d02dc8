"""protogalaxy::fold (src/folding.rs:14-75) on the device
(effsc_protogalaxy_fold) against the oracle: the reference's own cases
(two polynomials, four constants, random against the naive fold), both
fields, sizes that take one, two and three shared-memory passes, polynomials
too wide for a shared-memory group (per-level kernel), sizes wide enough for
the warp-subtree first pass, ragged counts and
level counts, trailing zeros, and inputs in device and pinned memory."""
import random

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


def rand_case(rng, n, width, levels, field):
    polys = np.array([[rng.randrange(O.P) for _ in range(width * field)] for _ in range(n)],
                     dtype=np.uint64).reshape(n, width, field)
    pairs = [tuple(np.array([rng.randrange(O.P) for _ in range(field)], dtype=np.uint64) for _ in range(2))
             for _ in range(levels)]
    return polys, pairs


def oracle_fold(pairs, polys, field):
    got = O.protogalaxy_fold(pairs, [p for p in polys])
    return got[:, 0] if field == 1 else got


def gpu_fold(E, pairs, polys, field):
    arr = polys[:, :, 0] if field == 1 else polys
    return E.protogalaxy_fold(pairs, np.ascontiguousarray(arr), field=field)


def test_two_polys(E):
    r = E.protogalaxy_fold([(3, 5)], [[1], [0, 1]])
    assert [int(x) for x in r] == [(1 - 3) % O.P, (3 - 5) % O.P, 5]


def test_four_polys(E):
    r = E.protogalaxy_fold([(1, 0)] * 2, [[1], [2], [3], [4]])
    assert [int(x) for x in r] == [4]


@pytest.mark.parametrize("field", [1, 3])
def test_matches_naive(E, field):
    rng = random.Random(field)
    polys, pairs = rand_case(rng, 8, 3, 3, field)
    want = R.protogalaxy_fold_naive([(tuple(int(x) for x in R_pad(a)), tuple(int(x) for x in R_pad(b)))
                                     for a, b in pairs],
                                    [[tuple(int(x) for x in R_pad(c)) for c in p] for p in polys])
    got = gpu_fold(E, pairs, polys, field)
    got3 = [tuple(int(x) for x in R_pad(c)) for c in (got if field == 3 else got.reshape(-1, 1))]
    assert got3 == want


def R_pad(c):
    c = np.asarray(c, dtype=np.uint64).reshape(-1)
    return list(c) + [0] * (3 - c.size)


@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("n,width", [(2, 1), (4, 8), (64, 8), (1024, 8), (1 << 14, 4), (1 << 12, 30),
                                     (1 << 11, 100), (16, 700), (8, 2100), (4, 7000), (1 << 16, 1),
                                     (1 << 18, 2), (1 << 18, 8)])
def test_sizes_match_oracle(E, field, n, width):
    rng = random.Random(n * 7 + width + field)
    levels = n.bit_length() - 1
    if n * width > (1 << 16):     # keep the generator and the oracle quick
        polys = np.asarray(O.gen_table(n * 131 + width, n * width * field), dtype=np.uint64).reshape(n, width, field)
        pairs = [tuple(np.array(O.gen_table(1000 + 2 * k + h, field), dtype=np.uint64) for h in range(2))
                 for k in range(levels)]
    else:
        polys, pairs = rand_case(rng, n, width, levels, field)
    assert np.array_equal(gpu_fold(E, pairs, polys, field), oracle_fold(pairs, polys, field))


@pytest.mark.parametrize("field", [1, 3])
@pytest.mark.parametrize("n,levels", [(0, 2), (1, 3), (3, 1), (3, 2), (5, 2), (6, 3), (4, 0), (4, 1), (2, 5),
                                      (100, 7), (1000, 4)])
def test_ragged_counts_and_levels(E, field, n, levels):
    rng = random.Random(n * 13 + levels)
    polys, pairs = rand_case(rng, max(n, 1), 3, levels, field)
    polys = polys[:n]
    got = gpu_fold(E, pairs, polys, field) if n else E.protogalaxy_fold(pairs, [], field=field)
    want = oracle_fold(pairs, polys, field) if n else O.protogalaxy_fold(pairs, [])
    assert np.array_equal(np.asarray(got).reshape(want.shape), want)


@pytest.mark.parametrize("field", [1, 3])
def test_trailing_zeros_and_zero_result(E, field):
    rng = random.Random(77)
    polys, pairs = rand_case(rng, 8, 6, 3, field)
    polys[:, 3:, :] = 0                       # degree 2 stored in width 6
    got = gpu_fold(E, pairs, polys, field)
    assert np.array_equal(got, oracle_fold(pairs, polys, field))
    assert len(got) == 3 + 3
    same = np.repeat(polys[:1], 8, axis=0)    # all differences zero: the first polynomial
    assert np.array_equal(gpu_fold(E, pairs, same, field), oracle_fold(pairs, same, field))
    zero = np.zeros_like(polys)
    assert len(gpu_fold(E, pairs, zero, field)) == 1    # the zero polynomial as one term
    one = polys[:1].copy()
    one[0, 1:, :] = 0
    assert len(gpu_fold(E, pairs, one, field)) == 1      # a lone input comes back as itself
    assert len(gpu_fold(E, pairs, np.zeros_like(one), field)) == 0


def test_device_and_pinned_inputs(E):
    import torch
    n, width, field = 1 << 12, 8, 3
    polys = np.asarray(O.gen_table(5, n * width * field), dtype=np.uint64).reshape(n, width, field)
    pairs = [tuple(np.array(O.gen_table(50 + 2 * k + h, field), dtype=np.uint64) for h in range(2))
             for k in range(12)]
    want = oracle_fold(pairs, polys, field)
    host = torch.from_numpy(polys.view(np.int64).reshape(-1).copy())
    dev = host.to("cuda")
    pinned = host.pin_memory()
    for t in (dev, pinned):
        got = E.protogalaxy_fold_raw(pairs, t.data_ptr(), n, width, field=field)
        assert np.array_equal(got, want)


def test_rejects(E):
    import ctypes
    from effsc_gpu import _lib
    L = E.load()
    ctx = E.Context.default()
    out = np.zeros(8, dtype=np.uint64)
    n_out = ctypes.c_size_t(0)
    polys = np.ones(4, dtype=np.uint64)
    pairs = np.ones(4, dtype=np.uint64)
    p = lambda a: a.ctypes.data_as(_lib.u64p)  # noqa: E731
    assert L.effsc_protogalaxy_fold(ctx.h, 2, p(pairs), 1, p(polys), 2, 2, p(out), ctypes.byref(n_out)) != 0
    assert L.effsc_protogalaxy_fold(ctx.h, 1, p(pairs), 1, p(polys), 2, 1 << 21, p(out), ctypes.byref(n_out)) != 0
    assert L.effsc_protogalaxy_fold(ctx.h, 1, None, 1, p(polys), 2, 2, p(out), ctypes.byref(n_out)) != 0
    with pytest.raises(ValueError):
        E.protogalaxy_fold([(1, 2)], [[1], [2]], field=2)
