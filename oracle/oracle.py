"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is the checker: the tests, the smoke check and the CPU-baseline leg
of ``bench.py`` use it to produce the expected proof for the same seeded
inputs.  It is never on the product path.

Field elements are numpy ``uint64`` arrays with a trailing axis of 3
(Fp3 AoS ``[c0, c1, c2]``, canonical residues); base-field values are the
embedded triples ``(x, 0, 0)``.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None

ML, IP, COEF, EQF, GKR = 0, 1, 2, 3, 4
MSB, LSB = 0, 1
P = 0xFFFFFFFF00000001
W = 0xFFFFFFF800000001

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.or_fp_add.restype = ctypes.c_uint64
        L.or_fp_add.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.or_fp_sub.restype = ctypes.c_uint64
        L.or_fp_sub.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.or_fp_mul.restype = ctypes.c_uint64
        L.or_fp_mul.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.or_fp_inv.restype = ctypes.c_uint64
        L.or_fp_inv.argtypes = [ctypes.c_uint64]
        L.or_fp_to_mont.restype = ctypes.c_uint64
        L.or_fp_to_mont.argtypes = [ctypes.c_uint64]
        L.or_fp_from_mont.restype = ctypes.c_uint64
        L.or_fp_from_mont.argtypes = [ctypes.c_uint64]
        L.or_f3_mul.argtypes = [_u64p, _u64p, _u64p]
        L.or_splitmix64_mix.restype = ctypes.c_uint64
        L.or_splitmix64_mix.argtypes = [ctypes.c_uint64]
        L.or_table_seed.restype = ctypes.c_uint64
        L.or_table_seed.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.or_gen_element.restype = ctypes.c_uint64
        L.or_gen_element.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.or_gen_table.argtypes = [ctypes.c_uint64, ctypes.c_uint64, _u64p]
        L.or_keccak_f1600.argtypes = [_u64p]
        L.or_transcript_size.restype = ctypes.c_size_t
        L.or_transcript_init_keccak.argtypes = [ctypes.c_void_p, ctypes.c_int, _u8p, ctypes.c_size_t]
        L.or_transcript_init_test.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64]
        L.or_transcript_absorb.argtypes = [ctypes.c_void_p, _u8p, ctypes.c_size_t]
        L.or_transcript_squeeze.argtypes = [ctypes.c_void_p, _u8p, ctypes.c_size_t]
        L.or_transcript_send.argtypes = [ctypes.c_void_p, _u64p]
        L.or_transcript_challenge.argtypes = [ctypes.c_void_p, _u64p]
        L.or_prover_new.restype = ctypes.c_void_p
        L.or_prover_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(_u64p), ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]
        L.or_eqf_new.restype = ctypes.c_void_p
        L.or_eqf_new.argtypes = [ctypes.c_int, _u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, ctypes.c_int]
        L.or_gkr_new.restype = ctypes.c_void_p
        L.or_gkr_new.argtypes = [ctypes.c_int, _u64p, _u64p, _u64p, ctypes.c_size_t, ctypes.c_int]
        L.or_gkr_claimed_w_values.argtypes = [ctypes.c_void_p, _u64p]
        L.or_prover_free.argtypes = [ctypes.c_void_p]
        L.or_prover_degree.restype = ctypes.c_int
        L.or_prover_degree.argtypes = [ctypes.c_void_p]
        L.or_prover_round.restype = ctypes.c_int
        L.or_prover_round.argtypes = [ctypes.c_void_p, _u64p, _u64p, _u64p]
        L.or_prover_finalize.argtypes = [ctypes.c_void_p, _u64p]
        L.or_prover_final_value.argtypes = [ctypes.c_void_p, _u64p]
        L.or_prover_table_len.restype = ctypes.c_size_t
        L.or_prover_table_len.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_prover_read_table.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p]
        L.or_sumcheck.restype = ctypes.c_int
        L.or_sumcheck.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, _u8p, ctypes.c_size_t,
                                  ctypes.c_int, _u64p, _u64p, _u64p]
        L.or_verify.restype = ctypes.c_int
        L.or_verify.argtypes = [_u64p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p, _u8p,
                                ctypes.c_size_t, _u64p, _u64p, _u64p]
        L.or_build_eq_table.argtypes = [_u64p, ctypes.c_size_t, _u64p]
        L.or_mle_eval_msb.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, _u64p]
        L.or_pg_fold.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                 _u64p, ctypes.POINTER(ctypes.c_size_t)]
        L.or_set_threads.argtypes = [ctypes.c_int]
        L.or_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_u64p)


def _bytes(b):
    b = bytes(b)
    buf = (ctypes.c_uint8 * max(1, len(b))).from_buffer_copy(b if b else b"\0")
    return buf, len(b)


def as_f(x):
    """One field element (scalar, 1 word or 3 words) as a (3,) uint64 triple."""
    a = np.asarray(x, dtype=np.uint64).reshape(-1)
    z = np.zeros(3, dtype=np.uint64)
    z[: a.size] = a
    return z


def as_table(x):
    """A table: 1-D arrays are base-field values, (n, 3) arrays Fp3 triples."""
    a = np.asarray(x, dtype=np.uint64)
    if a.ndim == 1:
        z = np.zeros((a.shape[0], 3), dtype=np.uint64)
        z[:, 0] = a
        return z
    assert a.ndim == 2 and a.shape[1] == 3, a.shape
    return np.ascontiguousarray(a)


def gen_table(seed, n):
    out = np.empty(n, dtype=np.uint64)
    lib().or_gen_table(seed, n, _p(out))
    return out


def table_seed(seed, t):
    return int(lib().or_table_seed(seed, t))


def set_threads(n):
    lib().or_set_threads(n)


def get_threads():
    return int(lib().or_get_threads())


class Transcript:
    """Keccak duplex transcript (kind 'keccak') or the seeded test transcript."""

    def __init__(self, deg, label=None, seed=None):
        L = lib()
        self.buf = ctypes.create_string_buffer(L.or_transcript_size())
        self.deg = deg
        if seed is not None:
            L.or_transcript_init_test(self.buf, deg, seed)
        else:
            b, n = _bytes(label if label is not None else b"")
            L.or_transcript_init_keccak(self.buf, deg, b, n)

    def absorb(self, data):
        b, n = _bytes(data)
        lib().or_transcript_absorb(self.buf, b, n)

    def squeeze(self, n):
        out = (ctypes.c_uint8 * n)()
        lib().or_transcript_squeeze(self.buf, out, n)
        return bytes(out)

    def send(self, v):
        v = as_f(v)
        lib().or_transcript_send(self.buf, _p(v))

    def challenge(self):
        out = np.zeros(3, dtype=np.uint64)
        lib().or_transcript_challenge(self.buf, _p(out))
        return out

    def state_bytes(self):
        return bytes(self.buf.raw)


def sha3_256(msg):
    """SHA3-256 built from the transcript's sponge primitives (raw state, no label)."""
    L = lib()
    buf = ctypes.create_string_buffer(L.or_transcript_size())
    # kind 0 = keccak, zero state; absorb/squeeze with SHA3 padding on the switch
    b, n = _bytes(msg)
    L.or_transcript_absorb(buf, b, n)
    out = (ctypes.c_uint8 * 32)()
    L.or_transcript_squeeze(buf, out, 32)
    return bytes(out)


class Prover:
    def __init__(self, kind, order, deg, tables, _handle=None):
        L = lib()
        self.kind, self.order, self.deg = kind, order, deg
        if _handle is not None:
            self.h = _handle
            return
        raw = [np.asarray(t, dtype=np.uint64) for t in tables]
        if all(r.ndim == 1 for r in raw):
            arrs = [np.ascontiguousarray(r) for r in raw]
            ncomp = 1
        else:
            # every table as (n, 3) triples, so base and Fp3 tables can be mixed
            arrs = [as_table(t) for t in raw]
            ncomp = 3
        ptrs = (_u64p * len(arrs))(*[_p(a) for a in arrs])
        lens = (ctypes.c_size_t * len(arrs))(*[a.shape[0] for a in arrs])
        self._keep = arrs
        self.h = L.or_prover_new(kind, order, deg, len(arrs), ptrs, lens, ncomp)

    @classmethod
    def eq_factored(cls, deg, w, p):
        w = as_table(w) if np.asarray(w).size else np.zeros((0, 3), dtype=np.uint64)
        p = np.ascontiguousarray(np.asarray(p, dtype=np.uint64))
        ncomp = 3 if p.ndim == 2 else 1
        h = lib().or_eqf_new(deg, _p(w), w.shape[0], _p(p), p.shape[0], ncomp)
        obj = cls(EQF, MSB, deg, None, _handle=h)
        return obj

    @classmethod
    def gkr(cls, deg, add, mult, w):
        """GkrProver (src/provers/gkr.rs): add, mult of n*n, w of n elements."""
        raw = [np.asarray(t, dtype=np.uint64) for t in (add, mult, w)]
        if all(r.ndim == 1 for r in raw):
            arrs, ncomp = [np.ascontiguousarray(r) for r in raw], 1
        else:
            arrs, ncomp = [as_table(r) for r in raw], 3
        h = lib().or_gkr_new(deg, _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), arrs[2].shape[0], ncomp)
        obj = cls(GKR, MSB, deg, None, _handle=h)
        obj._keep = arrs
        return obj

    def claimed_w_values(self):
        out = np.zeros((2, 3), dtype=np.uint64)
        lib().or_gkr_claimed_w_values(self.h, _p(out))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_prover_free(self.h)
            self.h = None

    def degree(self):
        return int(lib().or_prover_degree(self.h))

    def round(self, chal=None, aux=False):
        d = self.degree()
        out = np.zeros((max(d, 1), 3), dtype=np.uint64)
        ax = np.zeros((2, 3), dtype=np.uint64)
        c = as_f(chal) if chal is not None else None
        rc = lib().or_prover_round(self.h, _p(c) if c is not None else None, _p(out), _p(ax))
        if rc:
            raise ValueError("oracle prover rejected the round (the reference panics here)")
        return (out, ax) if aux else out

    def finalize(self, chal):
        c = as_f(chal)
        lib().or_prover_finalize(self.h, _p(c))

    def final_value(self):
        out = np.zeros(3, dtype=np.uint64)
        lib().or_prover_final_value(self.h, _p(out))
        return out

    def table(self, i):
        n = int(lib().or_prover_table_len(self.h, i))
        out = np.zeros((n, 3), dtype=np.uint64)
        if n:
            lib().or_prover_read_table(self.h, i, _p(out))
        return out


def sumcheck(prover, num_rounds, transcript, hook=b"", legacy=False):
    """Runner (reference src/runner.rs:29-69).  Returns (round_polys, challenges, final)."""
    d = prover.degree()
    nsend = 2 if legacy else d
    rp = np.zeros((num_rounds, nsend, 3), dtype=np.uint64)
    ch = np.zeros((num_rounds, 3), dtype=np.uint64)
    fv = np.zeros(3, dtype=np.uint64)
    hb, hn = _bytes(hook)
    rc = lib().or_sumcheck(prover.h, num_rounds, transcript.buf, hb, hn, 1 if legacy else 0,
                           _p(rp), _p(ch), _p(fv))
    if rc:
        raise ValueError("oracle sumcheck failed (the reference panics here)")
    return rp, ch, fv


def verify(claimed_sum, degree, num_rounds, transcript, round_polys, hook=b""):
    """sumcheck_verify (reference src/verifier.rs:61-139).  Returns (challenges, final_claim)."""
    cs = as_f(claimed_sum)
    rp = np.ascontiguousarray(np.asarray(round_polys, dtype=np.uint64))
    ch = np.zeros((num_rounds, 3), dtype=np.uint64)
    fc = np.zeros(3, dtype=np.uint64)
    hb, hn = _bytes(hook)
    lib().or_verify(_p(cs), degree, num_rounds, transcript.buf, hb, hn, _p(rp), _p(ch), _p(fc))
    return ch, fc


def build_eq_table(w):
    w = as_table(w)
    v = w.shape[0]
    out = np.zeros((1 << v, 3), dtype=np.uint64)
    lib().or_build_eq_table(_p(w), v, _p(out))
    return out


def mle_eval_msb(table, point):
    t = as_table(table)
    pt = as_table(point)
    out = np.zeros(3, dtype=np.uint64)
    lib().or_mle_eval_msb(_p(t), t.shape[0], _p(pt), pt.shape[0], _p(out))
    return out


def protogalaxy_fold(pairs, polys):
    """protogalaxy::fold (reference src/folding.rs:14-75), release-build
    semantics.  pairs: (a, b) per level, field elements (1 or 3 words);
    polys: a list of coefficient arrays (ascending degree; 1 or 3 words per
    coefficient), or one zero-padded array of shape (n, width) (base field)
    or (n, width, 3).  Returns the trimmed coefficients as an (len, 3) array."""
    pr = np.zeros((max(len(pairs), 1), 2, 3), dtype=np.uint64)
    for k, (a, b) in enumerate(pairs):
        pr[k, 0], pr[k, 1] = as_f(a), as_f(b)
    if isinstance(polys, np.ndarray) and polys.ndim in (2, 3):
        buf = np.ascontiguousarray(polys, dtype=np.uint64)
        n, width = buf.shape[0], buf.shape[1]
        ncomp = 1 if buf.ndim == 2 else 3
    else:
        rows = [np.asarray(p, dtype=np.uint64).reshape(len(p), -1) if len(p) else np.zeros((0, 3), np.uint64)
                for p in polys]
        n = len(rows)
        width = max([r.shape[0] for r in rows] + [0])
        buf = np.zeros((max(n, 1), width, 3), dtype=np.uint64)
        for i, r in enumerate(rows):
            buf[i, :r.shape[0], :r.shape[1]] = r
        ncomp = 3
    out = np.zeros((width + len(pairs) + 1, 3), dtype=np.uint64)
    n_out = ctypes.c_size_t(0)
    lib().or_pg_fold(_p(pr), len(pairs), _p(buf) if buf.size else None, n, width, ncomp, _p(out),
                     ctypes.byref(n_out))
    return out[: n_out.value].copy()


def fp_mul(a, b):
    return int(lib().or_fp_mul(a, b))


def f3_mul(a, b):
    a, b = as_f(a), as_f(b)
    out = np.zeros(3, dtype=np.uint64)
    lib().or_f3_mul(_p(a), _p(b), _p(out))
    return out
