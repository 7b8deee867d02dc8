"""The round entry point that allocates no device memory.

effsc_ip_round_noalloc is for callers that cannot let this library call
cudaMalloc: applications whose own memory pool already holds the GPU's HBM,
and code sharing a stream with latency-critical work that a synchronising
allocation would stall.  The caller owns every buffer; the library's only
scratch is a static device array.  This test drives it through the C ABI on
caller-owned (torch) buffers, two calls in a row -- round 0, then a folding
round with an Fp3 challenge done in place -- and requires exactly the values
of the regular prover entry point (effsc_prover_round) on the same tables.
It sits in its own file, collected last, so a failure here never hides the
other tests of a run that stops at the first failure.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = 0xFFFFFFFF00000001


def test_noalloc_round_matches_prover_round_two_calls():
    import torch
    sys.path.insert(0, os.path.join(ROOT, "efficient-sumcheck_gb300"))
    import effsc_gpu as E
    from effsc_gpu import _lib
    L = E.load()

    n = 1 << 14
    rng = np.random.default_rng(0x0A110C)
    a = rng.integers(0, P, size=(n, 3), dtype=np.uint64)
    b = rng.integers(0, P, size=(n, 3), dtype=np.uint64)
    r = rng.integers(0, P, size=3, dtype=np.uint64)

    # caller-owned device memory, structure of arrays: c0[n], c1[n], c2[n]
    dev = torch.device("cuda", 0)
    da = torch.from_numpy(np.ascontiguousarray(a.T).reshape(-1).view(np.int64)).to(dev)
    db = torch.from_numpy(np.ascontiguousarray(b.T).reshape(-1).view(np.int64)).to(dev)
    out = torch.zeros(6, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    reference = E.InnerProductProver(a, b, field=E.FP3)

    # call 1: round 0 (no challenge)
    _lib.check(L.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), None, None, n, None,
                                        out.data_ptr(), 0, stream))
    torch.cuda.synchronize(dev)
    got0 = out.cpu().numpy().view(np.uint64).reshape(2, 3)
    assert (got0 == reference.round(None)).all()

    # call 2: fold with an Fp3 challenge in place, evaluate the next round
    chal = np.ascontiguousarray(r)
    _lib.check(L.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), da.data_ptr(), db.data_ptr(), n,
                                        chal.ctypes.data_as(_lib.u64p), out.data_ptr(), 0, stream))
    torch.cuda.synchronize(dev)
    got1 = out.cpu().numpy().view(np.uint64).reshape(2, 3)
    assert (got1 == reference.round(r)).all()

    # the folded tables sit in the first n/2 entries of each component array
    half = n // 2
    fa = da.cpu().numpy().view(np.uint64).reshape(3, n)[:, :half].T
    fb = db.cpu().numpy().view(np.uint64).reshape(3, n)[:, :half].T
    assert (fa == reference.table(0)).all()
    assert (fb == reference.table(1)).all()

    # a grid beyond the static scratch is refused before any GPU work
    with pytest.raises(E.EffscError):
        _lib.check(L.effsc_ip_round_noalloc(da.data_ptr(), db.data_ptr(), None, None, n, None,
                                            out.data_ptr(), 4097, stream))
