"""Failure handling without a GPU fault.

The only waits in the library's kernels are the TMA-staged round kernel's
waits on its own mbarriers; each gives up after a time limit, records
EFFSC_STATUS_TIMEOUT and returns.  The self-test entry point runs that wait on
a barrier nothing completes (short limit) and on one that completes: the
status must say so and the context must stay usable.  Host-side failures
(bad arguments, requests larger than the serving budget, reference panics)
are covered beside the features they guard."""
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TIMEOUT = 4


@pytest.fixture(scope="module")
def E():
    import effsc_gpu
    effsc_gpu.load()
    return effsc_gpu


def run_wait(E, limit_ns, arrive):
    import ctypes
    from effsc_gpu import _lib
    st = ctypes.c_uint32(123)
    _lib.check(E.load().effsc_diag_bounded_wait(E.Context.default().h, limit_ns, arrive, ctypes.byref(st)))
    return st.value


def test_wait_that_nothing_completes_gives_up(E):
    t0 = time.perf_counter()
    assert run_wait(E, 2_000_000, 0) == TIMEOUT
    assert time.perf_counter() - t0 < 5.0


def test_completed_wait_reports_ok(E):
    assert run_wait(E, 2_000_000, 1) == 0


def test_context_usable_after_timeout(E):
    assert run_wait(E, 1_000_000, 0) == TIMEOUT
    g = np.random.default_rng(1)
    a = g.integers(0, O.P, size=1 << 10, dtype=np.uint64)
    b = g.integers(0, O.P, size=1 << 10, dtype=np.uint64)
    proof = E.InnerProductProver(a, b).prove(10, E.Transcript.keccak(3, b"after"))
    rp, ch, fv = O.sumcheck(O.Prover(O.IP, O.MSB, 3, [a, b]), 10, O.Transcript(3, label=b"after"))
    assert np.array_equal(proof.round_polys, rp) and np.array_equal(proof.final_value, fv)


def test_limit_is_capped(E):
    with pytest.raises(E.EffscError):
        run_wait(E, 3_000_000_000, 0)
