"""The round entry point that allocates no device memory.

effsc_ip_round_noalloc is for callers that cannot let this library call
cudaMalloc: applications whose own memory pool already holds the GPU's HBM,
and code sharing a stream with latency-critical work that a synchronising
allocation would stall.  The caller owns every buffer; the library's only
scratch is a static device array.  These tests drive it through the C ABI on
caller-owned (torch) buffers, two calls in a row each, and require exactly
the values of the CPU oracle and of the regular prover entry point
(effsc_prover_round) on the same tables:
* power-of-two lengths (4, the smallest folding length, and 2^14): round 0,
  then a folding round with an Fp3 challenge, in place or into separate
  output buffers; the folded tables are compared too;
* other lengths (1, 3, 1000): round 0 with the MSB padding rule, twice (the
  second call must not see anything the first left in the shared scratch);
* grids of 1 block, the library's choice (0) and the scratch limit (4096).
The file is collected last, so a failure here never hides the other tests of
a run that stops at the first failure.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = 0xFFFFFFFF00000001
for _p in (ROOT, os.path.join(ROOT, "efficient-sumcheck_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def _setup(n, seed):
    import torch
    import effsc_gpu as E
    from effsc_gpu import _lib
    lib = E.load()
    rng = np.random.default_rng(seed)
    a = rng.integers(0, P, size=(n, 3), dtype=np.uint64)
    b = rng.integers(0, P, size=(n, 3), dtype=np.uint64)
    r = rng.integers(0, P, size=3, dtype=np.uint64)
    dev = torch.device("cuda", 0)
    # caller-owned device memory, structure of arrays: c0[n], c1[n], c2[n]
    da = torch.from_numpy(np.ascontiguousarray(a.T).reshape(-1).view(np.int64)).to(dev)
    db = torch.from_numpy(np.ascontiguousarray(b.T).reshape(-1).view(np.int64)).to(dev)
    out = torch.full((6,), -1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    return torch, E, _lib, lib, a, b, r, da, db, out, stream


def _evals(torch, out):
    torch.cuda.synchronize(out.device)
    return out.cpu().numpy().view(np.uint64).reshape(2, 3)


@pytest.mark.parametrize("blocks", [0, 1, 4096])
@pytest.mark.parametrize("inplace", [True, False])
@pytest.mark.parametrize("n", [4, 1 << 14])
def test_noalloc_fold_round_two_calls(n, inplace, blocks):
    from oracle import oracle as O
    torch, E, _lib, lib, a, b, r, da, db, out, stream = _setup(n, 0x0A110C + n + blocks + inplace)
    regular = E.InnerProductProver(a, b, field=E.FP3)
    orc = O.Prover(O.IP, O.MSB, 2, [a, b])

    # call 1: round 0 (no challenge)
    _lib.check(lib.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), None, None, n, None,
                                          out.data_ptr(), blocks, stream))
    got0 = _evals(torch, out)
    assert (got0 == orc.round(None)).all(), "round 0 differs from the oracle"
    assert (got0 == regular.round(None)).all(), "round 0 differs from effsc_prover_round"

    # call 2: fold with an Fp3 challenge (in place or out of place), evaluate the next round
    if inplace:
        oa, ob = da, db
    else:
        oa = torch.zeros_like(da)
        ob = torch.zeros_like(db)
    chal = np.ascontiguousarray(r)
    _lib.check(lib.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), oa.data_ptr(), ob.data_ptr(), n,
                                          chal.ctypes.data_as(_lib.u64p), out.data_ptr(), blocks, stream))
    got1 = _evals(torch, out)
    assert (got1 == orc.round(r)).all(), "folding round differs from the oracle"
    assert (got1 == regular.round(r)).all(), "folding round differs from effsc_prover_round"

    # the folded tables sit in the first n/2 entries of each component array
    half = n // 2
    fa = oa.cpu().numpy().view(np.uint64).reshape(3, n)[:, :half].T
    fb = ob.cpu().numpy().view(np.uint64).reshape(3, n)[:, :half].T
    assert (fa == orc.table(0)).all() and (fb == orc.table(1)).all(), "folded tables differ from the oracle"
    assert (fa == regular.table(0)).all() and (fb == regular.table(1)).all()
    if not inplace:
        # out of place: the inputs are untouched
        assert (da.cpu().numpy().view(np.uint64).reshape(3, n).T == a).all()
        assert (db.cpu().numpy().view(np.uint64).reshape(3, n).T == b).all()


@pytest.mark.parametrize("blocks", [0, 1, 4096])
@pytest.mark.parametrize("n", [1, 3, 1000])
def test_noalloc_round0_padded_lengths_two_calls(n, blocks):
    from oracle import oracle as O
    torch, E, _lib, lib, a, b, r, da, db, out, stream = _setup(n, 0x0A110D + n + blocks)
    want = O.Prover(O.IP, O.MSB, 2, [a, b]).round(None)
    assert (want == E.InnerProductProver(a, b, field=E.FP3).round(None)).all()
    for _ in range(2):
        out.fill_(-1)
        _lib.check(lib.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), None, None, n, None,
                                              out.data_ptr(), blocks, stream))
        assert (_evals(torch, out) == want).all(), "round 0 differs from the oracle"


def test_noalloc_rejects_before_gpu_work():
    torch, E, _lib, lib, a, b, r, da, db, out, stream = _setup(16, 1)
    # a grid beyond the static scratch
    with pytest.raises(E.EffscError):
        _lib.check(lib.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), None, None, 16, None,
                                              out.data_ptr(), 4097, stream))
    # a folding round on a length that is not a power of two >= 4
    chal = np.ascontiguousarray(r)
    for bad in (2, 12):
        with pytest.raises(E.EffscError):
            _lib.check(lib.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), da.data_ptr(), db.data_ptr(), bad,
                                                  chal.ctypes.data_as(_lib.u64p), out.data_ptr(), 0, stream))
