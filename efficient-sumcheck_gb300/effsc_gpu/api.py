"""Python mirror of the effsc crate API over the GPU C ABI.

Names, argument meaning and error behaviour follow the Rust crate
(compsec-epfl/efficient-sumcheck):

  * provers: MultilinearProver[LSB] (src/provers/multilinear*.rs),
    InnerProductProver[LSB] (src/provers/inner_product*.rs),
    CoefficientProver[LSB] with the device product evaluator
    (src/provers/coefficient*.rs), EqFactoredProver (src/provers/eq_factored.rs);
    each exposes degree() / round(challenge) / finalize(r) / final_value()
    (the SumcheckProver trait, src/sumcheck_prover.rs:36-71) and the
    reference's post-state accessors;
  * sumcheck(prover, num_rounds, transcript, hook) -- src/runner.rs:29-69;
  * SumcheckProof -- src/proof.rs:18-34;
  * sumcheck_verify -- src/verifier.rs:61-139;
  * fold -- src/fold.rs:14;
  * the legacy runners inner_product_sumcheck[_partial] and
    multilinear_sumcheck[_partial] (src/lib.rs:51-57).

Field elements are numpy uint64 arrays: an element of F = Fp is one word, an
element of F = Fp3 is three words [c0, c1, c2].  Tables are 1-D (base field,
the embedded elements) or (n, 3) arrays (Fp3).
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, load, u64p, vp

ML, IP, COEF, EQF, GKR = 0, 1, 2, 3, 4
MSB, LSB = 0, 1
FP, FP3 = 1, 3
CANONICAL, MONTGOMERY = 0, 1
T_KECCAK, T_TEST = 0, 1

P = 0xFFFFFFFF00000001


def _p(a):
    return a.ctypes.data_as(u64p)


def _bytes(b):
    b = bytes(b)
    buf = (ctypes.c_uint8 * max(1, len(b))).from_buffer_copy(b if b else b"\0")
    return buf, len(b)


class Context:
    """One GPU and one CUDA stream (effsc_ctx)."""
    _default = None

    def __init__(self, device=0):
        L = load()
        h = vp()
        check(L.effsc_ctx_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def synchronize(self):
        check(load().effsc_ctx_synchronize(self.h))

    def set_stream(self, stream_handle):
        check(load().effsc_ctx_set_stream(self.h, stream_handle))


def launch_count():
    return int(load().effsc_launch_count())


def launch_count_reset():
    load().effsc_launch_count_reset()


def _elem(v, field):
    """Coerce one field element to a uint64 array of `field` words."""
    a = np.ascontiguousarray(np.asarray(v, dtype=np.uint64).reshape(-1))
    if a.size == field:
        return a
    if a.size == 1 and field == 3:
        return np.array([a[0], 0, 0], dtype=np.uint64)
    if a.size == 3 and field == 1:
        if a[1] or a[2]:
            raise ValueError("Fp3 value for an Fp prover")
        return a[:1].copy()
    raise ValueError("bad field element shape %s" % (a.shape,))


# ---------------------------------------------------------------------------
# transcripts
# ---------------------------------------------------------------------------
class Transcript:
    """ProverTranscript / VerifierTranscript (src/transcript/transcript.rs)."""

    def __init__(self, field=FP3, label=b"", kind=T_KECCAK, seed=0, repr=CANONICAL, _h=None):
        self.field, self.repr, self.kind = field, repr, kind
        if _h is not None:
            self.h = _h
            return
        b, n = _bytes(label)
        h = vp()
        check(load().effsc_transcript_create(kind, field, repr, b, n, seed, ctypes.byref(h)))
        self.h = h

    @classmethod
    def keccak(cls, field, label, repr=CANONICAL):
        return cls(field, label, T_KECCAK, 0, repr)

    @classmethod
    def test(cls, field, seed, repr=CANONICAL):
        """SanityTranscript semantics (src/transcript/sanity.rs): no-op sends."""
        return cls(field, b"", T_TEST, seed, repr)

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.effsc_transcript_destroy(self.h)
            self.h = None

    def clone(self):
        h = vp()
        check(load().effsc_transcript_clone(self.h, ctypes.byref(h)))
        return Transcript(self.field, repr=self.repr, kind=self.kind, _h=h)

    def absorb(self, data):
        b, n = _bytes(data)
        check(load().effsc_transcript_absorb(self.h, b, n))

    def squeeze(self, n):
        out = (ctypes.c_uint8 * n)()
        check(load().effsc_transcript_squeeze(self.h, out, n))
        return bytes(out)

    def send(self, value):
        v = _elem(value, self.field)
        check(load().effsc_transcript_send(self.h, _p(v)))

    def challenge(self):
        out = np.zeros(self.field, dtype=np.uint64)
        check(load().effsc_transcript_challenge(self.h, _p(out)))
        return out


@dataclass
class SumcheckProof:
    """src/proof.rs:18-34 (EvalsInfty round polynomials)."""
    round_polys: np.ndarray   # (num_rounds, degree, field)
    challenges: np.ndarray    # (num_rounds, field)
    final_value: np.ndarray   # (field,)


# ---------------------------------------------------------------------------
# provers
# ---------------------------------------------------------------------------
def _as_table(t, field):
    a = np.ascontiguousarray(np.asarray(t, dtype=np.uint64))
    if a.ndim == 1:
        return a, 1
    if a.ndim == 2 and a.shape[1] == 3:
        if field != FP3:
            raise ValueError("Fp3 table for an Fp prover")
        return a, 3
    raise ValueError("table must be (n,) base words or (n, 3) Fp3 words")


class _Prover:
    kind = None
    order = MSB

    def __init__(self, tables, field=FP3, repr=CANONICAL, ctx=None, _h=None):
        self.ctx = ctx or Context.default()
        self.field, self.repr = field, repr
        if _h is not None:
            self.h = _h
            return
        arrs = [_as_table(t, field) for t in tables]
        n = len(arrs)
        ptrs = (u64p * n)(*[_p(a) for a, _ in arrs])
        lens = (ctypes.c_size_t * n)(*[a.shape[0] for a, _ in arrs])
        nc = (ctypes.c_int * n)(*[c for _, c in arrs])
        h = vp()
        check(load().effsc_prover_create(self.ctx.h, self.kind, self.order, field, repr, n, ptrs, lens, nc,
                                         ctypes.byref(h)))
        self.h = h

    @classmethod
    def from_device(cls, dev_tables, lens, ncomp, field=FP3, ctx=None):
        """Construct on device-resident canonical SoA tables (not copied)."""
        ctx = ctx or Context.default()
        n = len(dev_tables)
        ptrs = (u64p * n)(*[ctypes.cast(ctypes.c_void_p(int(p)), u64p) for p in dev_tables])
        ls = (ctypes.c_size_t * n)(*lens)
        nc = (ctypes.c_int * n)(*ncomp)
        h = vp()
        check(load().effsc_prover_create_device(ctx.h, cls.kind, cls.order, field, n, ptrs, ls, nc, ctypes.byref(h)))
        obj = cls.__new__(cls)
        _Prover.__init__(obj, None, field, CANONICAL, ctx, _h=h)
        return obj

    @classmethod
    def from_host(cls, host_tables, field=FP3, ctx=None):
        """Construct over canonical tables left in host memory (numpy arrays,
        memory maps, pinned buffers) and read in place by the kernels; base
        tables are 1-D, Fp3 tables (n, 3) are passed as three component rows.
        The arrays are kept alive by the prover."""
        ctx = ctx or Context.default()
        keep = []
        ptrs, lens, ncomp = [], [], []
        for t in host_tables:
            a = np.asarray(t, dtype=np.uint64)
            if a.ndim == 2:
                a = np.ascontiguousarray(a.T)        # component-major (SoA)
                ncomp.append(3)
                lens.append(a.shape[1])
            else:
                if not (a.flags["C_CONTIGUOUS"]):
                    a = np.ascontiguousarray(a)
                ncomp.append(1)
                lens.append(a.shape[0])
            keep.append(a)
            ptrs.append(a.ctypes.data_as(u64p))
        n = len(keep)
        h = vp()
        check(load().effsc_prover_create_host(ctx.h, cls.kind, cls.order, field, n, (u64p * n)(*ptrs),
                                              (ctypes.c_size_t * n)(*lens), (ctypes.c_int * n)(*ncomp),
                                              ctypes.byref(h)))
        obj = cls.__new__(cls)
        _Prover.__init__(obj, None, field, CANONICAL, ctx, _h=h)
        obj._host_tables = keep
        return obj

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.effsc_prover_destroy(self.h)
            self.h = None

    def degree(self):
        return int(load().effsc_prover_degree(self.h))

    def round(self, challenge=None, aux=False):
        d = self.degree()
        out = np.zeros((d, self.field), dtype=np.uint64)
        ax = np.zeros((2, self.field), dtype=np.uint64)
        c = _elem(challenge, self.field) if challenge is not None else None
        check(load().effsc_prover_round(self.h, _p(c) if c is not None else None, _p(out), _p(ax)))
        return (out, ax) if aux else out

    def finalize(self, challenge):
        c = _elem(challenge, self.field)
        check(load().effsc_prover_finalize(self.h, _p(c)))

    def final_value(self):
        out = np.zeros(self.field, dtype=np.uint64)
        check(load().effsc_prover_final_value(self.h, _p(out)))
        return out

    def table_len(self, i):
        n = ctypes.c_size_t()
        check(load().effsc_prover_table_len(self.h, i, ctypes.byref(n)))
        return n.value

    def table(self, i):
        n = self.table_len(i)
        out = np.zeros((n, self.field), dtype=np.uint64)
        if n:
            check(load().effsc_prover_read_table(self.h, i, _p(out)))
        return out if self.field == FP3 else out.reshape(-1)

    def reset(self):
        check(load().effsc_prover_reset(self.h))

    def set_first_rounds(self, fused):
        """prove(): how the first rounds read the base tables.  False / 0: one
        pass per round; 1: rounds 0-2 of an InnerProduct, Multilinear or
        GkrProver proof in two passes; True / 2 (the default): as 1, and
        rounds 0-3 of an InnerProduct proof in two passes where they apply
        (Fp3 challenges, power-of-two base tables of 2^14 entries or more)."""
        level = 2 if fused is True else 0 if fused is False else int(fused)
        check(load().effsc_prover_set_first_rounds(self.h, level))

    def set_tail(self, max_len):
        """prove(): tables of at most max_len entries finish in the one-block
        tail kernel (None: as large as shared memory allows, 0: never)."""
        check(load().effsc_prover_set_tail(self.h, (1 << 64) - 1 if max_len is None else int(max_len)))

    def set_persistent(self, max_len):
        """prove(): InnerProduct rounds over Fp3 whose tables hold at most
        max_len entries run in one cooperative launch (0: never)."""
        check(load().effsc_prover_set_persistent(self.h, int(max_len)))

    def prove(self, num_rounds, transcript, hook=b"", use_graph=True):
        """Whole protocol on the device (effsc_prove) with the device transcript."""
        d = self.degree()
        rp = np.zeros((num_rounds, d, self.field), dtype=np.uint64)
        ch = np.zeros((num_rounds, self.field), dtype=np.uint64)
        fv = np.zeros(self.field, dtype=np.uint64)
        hb, hn = _bytes(hook)
        check(load().effsc_prove(self.h, num_rounds, transcript.h, hb, hn, 1 if use_graph else 0,
                                 _p(rp), _p(ch), _p(fv)))
        return SumcheckProof(rp, ch, fv)


class MultilinearProver(_Prover):
    """src/provers/multilinear.rs:25-80."""
    kind, order = ML, MSB

    def __init__(self, evals, field=FP3, repr=CANONICAL, ctx=None):
        super().__init__([evals], field, repr, ctx)

    def evals(self):
        return self.table(0)

    def num_variables(self):
        n = self.table_len(0)
        return 0 if n == 0 else (n - 1).bit_length()


class MultilinearProverLSB(MultilinearProver):
    """src/provers/multilinear_lsb.rs:29-194."""
    kind, order = ML, LSB


class InnerProductProver(_Prover):
    """src/provers/inner_product.rs:26-127."""
    kind, order = IP, MSB

    def __init__(self, a, b, field=FP3, repr=CANONICAL, ctx=None):
        super().__init__([a, b], field, repr, ctx)

    def evaluations(self):
        return self.table(0), self.table(1)

    def final_evaluations(self):
        if self.table_len(0) == 1:
            return self.table(0)[0], self.table(1)[0]
        z = np.zeros(self.field, dtype=np.uint64)
        return z, z.copy()


class InnerProductProverLSB(InnerProductProver):
    """src/provers/inner_product_lsb.rs:25-178."""
    kind, order = IP, LSB


class _Term(ctypes.Structure):
    _fields_ = [("coeff", ctypes.c_uint32), ("n_factors", ctypes.c_uint32),
                ("factors", ctypes.c_uint32 * 4), ("k", ctypes.c_uint64 * 3)]


def pw_even(i):
    """Factor: the even (lo) element of pairwise table i."""
    return ("pw", i, 0, 0)


def pw_odd(i):
    return ("pw", i, 0, 1)


def tw_even(t, col):
    """Factor: column `col` of the even (lo) row of tablewise table t."""
    return ("tw", t, col, 0)


def tw_odd(t, col):
    return ("tw", t, col, 1)


class Evaluator:
    """A declarative RoundPolyEvaluator (src/coefficient_sumcheck.rs:50-76):
    accumulate_pair adds, for every term (coeff, k, factors), k times the
    product of the factors into coefficient `coeff`.  Factors are pw_even(i),
    pw_odd(i), tw_even(t, c), tw_odd(t, c); k is a field element (an int, or
    3 words for Fp3), in the prover's representation."""

    def __init__(self, degree, terms):
        self.deg = int(degree)
        self.terms = [(int(c), k, list(f)) for c, k, f in terms]

    def degree(self):
        return self.deg

    def _program(self, n_pairwise, widths, field):
        base = [0]
        for w in widths:
            base.append(base[-1] + w)
        arr = (_Term * max(1, len(self.terms)))()
        for i, (c, k, fs) in enumerate(self.terms):
            arr[i].coeff = c
            arr[i].n_factors = len(fs)
            for j, (kind, t, col, odd) in enumerate(fs):
                column = t if kind == "pw" else n_pairwise + base[t] + col
                arr[i].factors[j] = 2 * column + odd
            kv = _elem(k, field)
            for j in range(field):
                arr[i].k[j] = int(kv[j])
        return arr


class CoefficientProver(_Prover):
    """src/provers/coefficient.rs:18-330.  Without `evaluator`: the device
    product evaluator -- accumulate_pair adds the coefficients of
    prod_i (lo_i + x (hi_i - lo_i)) over the pairwise tables (1 to 3 of them;
    degree = number of tables).  With `evaluator` (an Evaluator) and optional
    `tablewise` tables (each an (n, w) array of rows, or (n, w, 3) for Fp3):
    that evaluator over pairwise and tablewise tables; table(i) reads column i
    (the pairwise tables, then every tablewise column)."""
    kind, order = COEF, MSB

    def __init__(self, pairwise, field=FP3, repr=CANONICAL, ctx=None, evaluator=None, tablewise=()):
        if evaluator is None and not len(tablewise):
            super().__init__(list(pairwise), field, repr, ctx)
            self.n_pairwise = len(pairwise)
            return
        if evaluator is None:
            raise ValueError("tablewise tables need an evaluator")
        self.ctx = ctx or Context.default()
        self.field, self.repr = field, repr
        self.evaluator = evaluator
        pws = [_as_table(t, field) for t in pairwise]
        tws, widths, tnc = [], [], []
        for t in tablewise:
            a = np.ascontiguousarray(np.asarray(t, dtype=np.uint64))
            if a.ndim == 2:
                tnc.append(1)
            elif a.ndim == 3 and a.shape[2] == 3 and field == FP3:
                tnc.append(3)
            else:
                raise ValueError("tablewise table must be (n, w) or (n, w, 3)")
            tws.append(a)
            widths.append(a.shape[1])
        lens = {a.shape[0] for a, _ in pws} | {a.shape[0] for a in tws}
        if len(lens) != 1:
            raise ValueError("every table must have the same number of entries / rows")
        n = lens.pop()
        prog = evaluator._program(len(pws), widths, field)
        np_, nt = len(pws), len(tws)
        h = vp()
        check(load().effsc_coef_expr_create(
            self.ctx.h, self.order, field, repr, evaluator.degree(), np_,
            (u64p * max(np_, 1))(*[_p(a) for a, _ in pws]), (ctypes.c_int * max(np_, 1))(*[c for _, c in pws]), nt,
            (u64p * max(nt, 1))(*[_p(a) for a in tws]), (ctypes.c_size_t * max(nt, 1))(*widths),
            (ctypes.c_int * max(nt, 1))(*tnc), n, ctypes.cast(prog, vp), len(evaluator.terms), ctypes.byref(h)))
        self.h = h
        self.n_pairwise = np_
        self._keep = (pws, tws)

    def pairwise(self):
        return [self.table(i) for i in range(self.n_pairwise)]


class CoefficientProverLSB(CoefficientProver):
    """src/provers/coefficient_lsb.rs:37-237."""
    kind, order = COEF, LSB


class EqFactoredProver(_Prover):
    """src/provers/eq_factored.rs:67-289.  Tables: 0 = p, 1 = eq_l, 2 = eq_r."""
    kind, order = EQF, MSB

    def __init__(self, w, p, field=FP3, repr=CANONICAL, ctx=None):
        self.ctx = ctx or Context.default()
        self.field, self.repr = field, repr
        w = np.ascontiguousarray(np.asarray(w, dtype=np.uint64))
        if field == FP3 and w.ndim == 1:
            w3 = np.zeros((w.shape[0], 3), dtype=np.uint64)
            w3[:, 0] = w
            w = w3
        v = w.shape[0]
        pa, nc = _as_table(p, field)
        h = vp()
        check(load().effsc_eqf_create(self.ctx.h, field, repr, _p(np.ascontiguousarray(w.reshape(-1))), v,
                                      _p(pa), pa.shape[0], nc, ctypes.byref(h)))
        self.h = h

    def final_factors(self):
        if self.table_len(0) != 1:
            z = np.zeros(self.field, dtype=np.uint64)
            return z, z.copy()
        from .field import f_mul
        p0 = self.table(0)[0]
        e = f_mul(self.table(1)[0], self.table(2)[0], self.field, self.repr)
        return p0, e


# ---------------------------------------------------------------------------
# runner, verifier, free functions
# ---------------------------------------------------------------------------
class GkrProver(_Prover):
    """src/provers/gkr.rs:41-208.  add_evals, mult_evals: n*n elements;
    w_evals: n elements (n a power of two).  Tables: 0 = add, 1 = mult,
    2 = W_b, 3 = W_c (the witness, compact)."""
    kind, order = GKR, MSB

    def __init__(self, add_evals, mult_evals, w_evals, field=FP3, repr=CANONICAL, ctx=None):
        self.ctx = ctx or Context.default()
        self.field, self.repr = field, repr
        arrs = [_as_table(t, field) for t in (add_evals, mult_evals, w_evals)]
        nc = max(c for _, c in arrs)
        if nc == 3:
            arrs = [(a if c == 3 else np.stack([a, np.zeros_like(a), np.zeros_like(a)], axis=1), 3) for a, c in arrs]
        (ad, _), (mu, _), (w, _) = arrs
        n = w.shape[0]
        if ad.shape[0] != n * n or mu.shape[0] != n * n:
            raise AssertionError("add_evals and mult_evals must have len w^2")   # the reference asserts
        h = vp()
        check(load().effsc_gkr_create(self.ctx.h, field, repr, _p(np.ascontiguousarray(ad)),
                                      _p(np.ascontiguousarray(mu)), _p(np.ascontiguousarray(w)), n, nc,
                                      ctypes.byref(h)))
        self.h = h

    def claimed_w_values(self):
        out = np.zeros((2, self.field), dtype=np.uint64)
        check(load().effsc_gkr_claimed_w_values(self.h, _p(out)))
        return out


def sumcheck(prover, num_rounds, transcript, hook=None):
    """runner::sumcheck (src/runner.rs:29-69) on the host, one prover round per
    C-ABI call.  hook(round, transcript) runs after the round's messages."""
    d = prover.degree()
    f = prover.field
    rps = np.zeros((num_rounds, d, f), dtype=np.uint64)
    chs = np.zeros((num_rounds, f), dtype=np.uint64)
    prev = None
    for r in range(num_rounds):
        evals = prover.round(prev)
        for v in evals:
            transcript.send(v)
        rps[r] = evals
        if hook is not None:
            hook(r, transcript)
        prev = transcript.challenge()
        chs[r] = prev
    if prev is not None:
        prover.finalize(prev)
    return SumcheckProof(rps, chs, prover.final_value())


@dataclass
class CoefficientSumcheck:
    """Legacy return type, src/coefficient_sumcheck.rs:11-15: every round's
    polynomial in coefficient form (degree + 1 coefficients) and challenges."""
    prover_messages: list
    verifier_messages: list


def _coefficients(wire, aux, d, field, repr):
    """The round polynomial's coefficients c0..cd from the EvalsInfty wire and
    the (c0, c1) pair: c_d = h(inf); for degree 3, c2 from h(2)."""
    from .field import f_add, f_sub, f_mul, f_scale
    c0, c1 = aux[0], aux[1]
    if d <= 1:
        return [c0] if d == 0 else [c0, c1]
    if d == 2:
        return [c0, c1, wire[1]]
    c3 = wire[1]
    # h(2) = c0 + 2 c1 + 4 c2 + 8 c3
    t = f_sub(f_sub(f_sub(wire[2], c0, field, repr), f_scale(c1, 2, field, repr), field, repr),
              f_scale(c3, 8, field, repr), field, repr)
    return [c0, c1, f_scale(t, None, field, repr, inv=4), c3]


def coefficient_sumcheck(evaluator, tablewise, pairwise, n_rounds, transcript, field=FP3, repr=CANONICAL):
    """src/coefficient_sumcheck.rs:255-365: pairs (2k, 2k+1); each round sends
    the first `degree` coefficients of the round polynomial (the leading one
    is omitted), squeezes the challenge and reduces every table with it.
    Returns CoefficientSumcheck and the prover (its tables are the reduced
    tables)."""
    pr = CoefficientProverLSB(pairwise, field=field, repr=repr, evaluator=evaluator, tablewise=tablewise)
    d = evaluator.degree()
    msgs, chals, prev = [], [], None
    for _ in range(n_rounds):
        wire, aux = pr.round(prev, aux=True)
        coeffs = _coefficients(wire, aux, d, field, repr)
        for c in coeffs[:d]:
            transcript.send(c)
        msgs.append(np.array(coeffs, dtype=np.uint64).reshape(len(coeffs), field))
        prev = transcript.challenge()
        chals.append(prev)
    if prev is not None:
        pr.finalize(prev)
    return CoefficientSumcheck(msgs, chals), pr


def noop_hook(_round, _transcript):
    """src/lib.rs:28-33."""


def sumcheck_verify(claimed_sum, degree, num_rounds, transcript, round_polys, hook=b""):
    """src/verifier.rs:61-139.  Returns (challenges, final_claim)."""
    f = transcript.field
    cs = _elem(claimed_sum, f)
    rp = np.ascontiguousarray(np.asarray(round_polys, dtype=np.uint64))
    ch = np.zeros((num_rounds, f), dtype=np.uint64)
    fc = np.zeros(f, dtype=np.uint64)
    hb, hn = _bytes(hook)
    check(load().effsc_verify(f, transcript.repr, _p(cs), degree, num_rounds, transcript.h, hb, hn,
                              _p(rp) if rp.size else None, _p(ch), _p(fc)))
    return ch, fc


def protogalaxy_fold(coeffs, polys, field=FP, ctx=None):
    """protogalaxy::fold (src/folding.rs:14-75) on the device.  coeffs: the
    (a, b) pairs, one per level; polys: a list of coefficient arrays
    (ascending degree; `field` words per coefficient) or one zero-padded
    array of shape (n, width) for Fp, (n, width, 3) for Fp3 (for device
    memory see `protogalaxy_fold_raw`).  Returns the coefficients of the
    result, trailing zeros trimmed, shape (len,) for Fp and (len, 3) for
    Fp3."""
    ctx = ctx or Context.default()
    pairs = [(_elem(a, field), _elem(b, field)) for a, b in coeffs]
    if isinstance(polys, np.ndarray) and polys.ndim == (2 if field == 1 else 3):
        n, width = polys.shape[0], polys.shape[1]
        buf = np.ascontiguousarray(polys.astype(np.uint64, copy=False))
    else:
        rows = [np.asarray(p, dtype=np.uint64).reshape(-1, field) for p in polys]
        n = len(rows)
        width = max([r.shape[0] for r in rows] + [0])
        buf = np.zeros((max(n, 1), max(width, 1) * field), dtype=np.uint64)
        for i, r in enumerate(rows):
            buf[i, :r.shape[0] * field] = r.reshape(-1)
    return protogalaxy_fold_raw(pairs, buf.ctypes.data, n, width, field, ctx)


def protogalaxy_fold_raw(pairs, polys_ptr, n, width, field=FP, ctx=None):
    """The same on a raw pointer to n x width coefficients (device, pinned or
    host memory); pairs as (a, b) tuples of `field`-word arrays."""
    ctx = ctx or Context.default()
    pr = np.zeros((max(len(pairs), 1), 2, field), dtype=np.uint64)
    for k, (a, b) in enumerate(pairs):
        pr[k, 0], pr[k, 1] = _elem(a, field), _elem(b, field)
    out = np.zeros((max(width + len(pairs), 1), field), dtype=np.uint64)
    n_out = ctypes.c_size_t(0)
    check(load().effsc_protogalaxy_fold(ctx.h, field, _p(pr), len(pairs),
                                        ctypes.cast(polys_ptr, u64p) if polys_ptr else None, n, width, _p(out),
                                        ctypes.byref(n_out)))
    res = out[: n_out.value]
    return res.reshape(-1) if field == 1 else res.copy()


def sumcheck_verify_batch(claimed_sums, degree, round_polys, transcripts, hook=b"", field=FP3, ctx=None):
    """sumcheck_verify (src/verifier.rs:61-139) for many proofs on the device.
    round_polys: one array per proof of shape (rounds, max(degree, 1), field)
    or (rounds, degree, field); transcripts: one per proof at its starting
    state.  Returns (final_claims (n, field), challenges per proof)."""
    ctx = ctx or Context.default()
    n = len(round_polys)
    nw = max(int(degree), 1)
    rounds = [int(np.asarray(rp).shape[0]) for rp in round_polys]
    flat = np.ascontiguousarray(np.concatenate(
        [np.asarray(rp, dtype=np.uint64).reshape(-1) for rp in round_polys]) if n and sum(rounds)
        else np.zeros(1, dtype=np.uint64))
    cs = np.ascontiguousarray(np.asarray(claimed_sums, dtype=np.uint64).reshape(n, field))
    fin = np.zeros((n, field), dtype=np.uint64)
    ch = np.zeros((max(1, sum(rounds)), field), dtype=np.uint64)
    hb, hn = _bytes(hook)
    check(load().effsc_verify_batch(ctx.h, field, n, _p(cs), int(degree), (ctypes.c_uint32 * max(n, 1))(*rounds),
                                    (vp * max(n, 1))(*[t.h for t in transcripts]), hb, hn, _p(flat), _p(ch),
                                    _p(fin)))
    offs = np.concatenate([[0], np.cumsum(rounds)])
    return fin, [ch[offs[i]:offs[i + 1]] for i in range(n)]


def fold(values, weight, field=FP3, repr=CANONICAL, ctx=None):
    """effsc::fold (src/fold.rs:14): half-split fold with implicit zero padding."""
    ctx = ctx or Context.default()
    a, nc = _as_table(values, field)
    w = _elem(weight, field)
    n = a.shape[0]
    out = np.zeros((max(n, 1), field), dtype=np.uint64)
    ol = ctypes.c_size_t()
    check(load().effsc_fold(ctx.h, field, repr, _p(a), n, nc, _p(w), _p(out), ctypes.byref(ol)))
    out = out[: ol.value]
    return out if field == FP3 else out.reshape(-1)


def compute_sumcheck_polynomial(values, field=FP3, repr=CANONICAL, ctx=None):
    """src/multilinear_sumcheck.rs:86-124: (s0, s1) of a half-split table with
    implicit zero padding (s0 = low half plus the unpaired tail, s1 = high half)."""
    ctx = ctx or Context.default()
    a, nc = _as_table(values, field)
    out = np.zeros((2, field), dtype=np.uint64)
    check(load().effsc_compute_sumcheck_polynomial(ctx.h, field, repr, _p(a) if a.shape[0] else None, a.shape[0],
                                                   nc, _p(out)))
    return (out[0], out[1]) if field == FP3 else (out[0, 0], out[1, 0])


def fused_fold_and_compute_polynomial(values, weight, field=FP3, repr=CANONICAL, ctx=None):
    """src/multilinear_sumcheck.rs:189-254: the table folded by weight (as
    `fold`) and the folded table's (s0, s1).  The reference folds its Vec in
    place; here the folded table is returned: (folded, (s0, s1))."""
    ctx = ctx or Context.default()
    a, nc = _as_table(values, field)
    w = _elem(weight, field)
    n = a.shape[0]
    out = np.zeros((max(n, 1), field), dtype=np.uint64)
    ol = ctypes.c_size_t()
    s = np.zeros((2, field), dtype=np.uint64)
    check(load().effsc_fused_fold_and_compute_polynomial(ctx.h, field, repr, _p(a) if n else None, n, nc, _p(w),
                                                         _p(out), ctypes.byref(ol), _p(s)))
    out = out[: ol.value]
    folded = out if field == FP3 else out.reshape(-1)
    return folded, ((s[0], s[1]) if field == FP3 else (s[0, 0], s[1, 0]))


def build_eq_table(w, field=FP3, repr=CANONICAL, ctx=None):
    """eq(w, .) over {0,1}^v, MSB layout (src/provers/eq_factored.rs:217-239)."""
    ctx = ctx or Context.default()
    w = np.ascontiguousarray(np.asarray(w, dtype=np.uint64).reshape(-1))
    v = w.size // field
    out = np.zeros(((1 << v), field), dtype=np.uint64)
    check(load().effsc_build_eq_table(ctx.h, field, repr, _p(w), v, _p(out)))
    return out if field == FP3 else out.reshape(-1)


class Batch:
    """Many independent MSB InnerProduct (kind=IP) or Multilinear (kind=ML)
    provers proved together (effsc_batch_*): one kernel per round for every
    instance still active, the whole protocol replayed as one CUDA graph.

    ``tables`` is a list per instance of base-field tables (IP: [a, b],
    ML: [v]), each of 2^num_vars canonical words; or pass ``seeds`` (a list per
    instance of per-table seeds) to generate gen_uniform tables on the device.
    Instance i's proof is the one runner::sumcheck (src/runner.rs:29-69)
    produces with num_vars[i] rounds, transcript i and no hook.
    """

    def __init__(self, kind, num_vars, tables=None, seeds=None, field=FP3, ctx=None):
        self.ctx = ctx or Context.default()
        self.kind, self.field = kind, field
        self.num_vars = [int(v) for v in num_vars]
        n = len(self.num_vars)
        ntab = 2 if kind == IP else 1
        self.ntab = ntab
        nv = (ctypes.c_uint32 * n)(*self.num_vars)
        tp = None
        sp = None
        keep = []
        if tables is not None:
            flat = []
            for i, ts in enumerate(tables):
                if len(ts) != ntab:
                    raise ValueError("instance %d: expected %d tables" % (i, ntab))
                for t in ts:
                    a = np.ascontiguousarray(np.asarray(t, dtype=np.uint64).reshape(-1))
                    if a.size != 1 << self.num_vars[i]:
                        raise ValueError("instance %d: table length %d != 2^%d" % (i, a.size, self.num_vars[i]))
                    keep.append(a)
                    flat.append(_p(a))
            tp = (u64p * len(flat))(*flat)
        else:
            sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))
            if sd.size != n * ntab:
                raise ValueError("need %d seeds" % (n * ntab))
            keep.append(sd)
            sp = _p(sd)
        h = vp()
        check(load().effsc_batch_create(self.ctx.h, kind, field, n, nv, tp, sp, ctypes.byref(h)))
        self.h = h
        self.rows = np.concatenate([[0], np.cumsum(self.num_vars)]).astype(np.int64)

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.effsc_batch_destroy(self.h)
            self.h = None

    def __len__(self):
        return len(self.num_vars)

    def degree(self):
        return 2 if self.kind == IP else 1

    def _tx_array(self, transcripts):
        if len(transcripts) != len(self):
            raise ValueError("one transcript per instance")
        return (vp * len(transcripts))(*[t.h for t in transcripts])

    def prove_raw(self, transcripts, use_graph=True, outputs=True):
        """Run the protocol; returns (round_polys, challenges, final_values) as
        flat arrays (rows concatenated in instance order) or None."""
        d, f, rows = self.degree(), self.field, int(self.rows[-1])
        if not outputs:
            check(load().effsc_batch_prove(self.h, self._tx_array(transcripts), 1 if use_graph else 0, None, None, None))
            return None
        rp = np.zeros((rows, d, f), dtype=np.uint64)
        ch = np.zeros((rows, f), dtype=np.uint64)
        fv = np.zeros((len(self), f), dtype=np.uint64)
        check(load().effsc_batch_prove(self.h, self._tx_array(transcripts), 1 if use_graph else 0,
                                       _p(rp), _p(ch), _p(fv)))
        return rp, ch, fv

    def prove(self, transcripts, use_graph=True):
        """One SumcheckProof per instance."""
        rp, ch, fv = self.prove_raw(transcripts, use_graph)
        return [SumcheckProof(rp[self.rows[i]:self.rows[i + 1]], ch[self.rows[i]:self.rows[i + 1]], fv[i])
                for i in range(len(self))]

    def set_quads_per_thread(self, q):
        check(load().effsc_batch_set_quads_per_thread(self.h, int(q)))

    def set_tail(self, max_len):
        """Tables of at most max_len entries finish in the one-block tail
        kernel (None: as large as shared memory allows, 0: never)."""
        check(load().effsc_batch_set_tail(self.h, (1 << 64) - 1 if max_len is None else int(max_len)))

    def tune(self, transcripts, cache_path=None):
        """Autotune quadruples per thread and the tail switch; returns
        (quads_per_thread, tail_len)."""
        c = ctypes.c_int()
        t = ctypes.c_uint64()
        path = cache_path.encode() if cache_path else None
        check(load().effsc_batch_tune(self.h, self._tx_array(transcripts), path, ctypes.byref(c), ctypes.byref(t)))
        return c.value, t.value

    def device_table(self, inst, t):
        out = u64p()
        check(load().effsc_batch_device_table(self.h, inst, t, ctypes.byref(out)))
        return ctypes.cast(out, ctypes.c_void_p).value


class Server:
    """A request loop with continuous batching (effsc_server_*): MSB
    InnerProduct (kind=IP) / Multilinear (kind=ML) proofs of any size, admitted
    FIFO while at most ``max_active`` are in flight and their device memory
    fits in ``hbm_budget`` bytes; every step is one kernel in which each
    admitted request advances one round.  Each proof equals the one
    runner::sumcheck (src/runner.rs:29-69) gives for that request alone."""

    def __init__(self, hbm_budget, max_active=64, ctx=None):
        self.ctx = ctx or Context.default()
        h = vp()
        check(load().effsc_server_create(self.ctx.h, int(hbm_budget), int(max_active), ctypes.byref(h)))
        self.h = h
        self._meta = {}

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.effsc_server_destroy(self.h)
            self.h = None

    def submit(self, kind, num_vars, transcript, tables=None, seeds=None, field=FP3):
        """Queue one request; returns its id.  ``tables``: host tables (kept
        alive by this object until the proof is taken) or ``seeds``."""
        ntab = 2 if kind == IP else 1
        tp = sp = None
        keep = []
        if tables is not None:
            arrs = [np.ascontiguousarray(np.asarray(t, dtype=np.uint64).reshape(-1)) for t in tables]
            if len(arrs) != ntab or any(a.size != 1 << num_vars for a in arrs):
                raise ValueError("expected %d tables of 2^%d words" % (ntab, num_vars))
            keep = arrs
            tp = (u64p * ntab)(*[_p(a) for a in arrs])
        else:
            sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))
            if sd.size < ntab:
                raise ValueError("need %d seeds" % ntab)
            keep = [sd]
            sp = _p(sd)
        rid = ctypes.c_uint64()
        check(load().effsc_server_submit(self.h, kind, field, int(num_vars), tp, sp, transcript.h, ctypes.byref(rid)))
        self._meta[rid.value] = (kind, field, int(num_vars), keep)
        return rid.value

    def progress(self, wait=False):
        """Admit, launch one step, collect finished proofs; returns the number
        of requests not yet taken."""
        n = ctypes.c_uint32()
        check(load().effsc_server_progress(self.h, 1 if wait else 0, ctypes.byref(n)))
        return n.value

    def take(self):
        """(id, SumcheckProof, queue_s, latency_s) of the oldest finished
        proof, or None."""
        rid = ctypes.c_uint64()
        nv = ctypes.c_uint32()
        rp = np.zeros((34, 2, 3), dtype=np.uint64)
        ch = np.zeros((34, 3), dtype=np.uint64)
        fv = np.zeros(3, dtype=np.uint64)
        qs = ctypes.c_double()
        ls = ctypes.c_double()
        check(load().effsc_server_take(self.h, ctypes.byref(rid), ctypes.byref(nv), _p(rp), _p(ch), _p(fv),
                                       ctypes.byref(qs), ctypes.byref(ls)))
        if rid.value == (1 << 64) - 1:
            return None
        kind, field, n, _ = self._meta.pop(rid.value)
        d = 2 if kind == IP else 1
        rpf = rp.reshape(-1)[:n * d * field].reshape(n, d, field).copy()
        chf = ch.reshape(-1)[:n * field].reshape(n, field).copy()
        return rid.value, SumcheckProof(rpf, chf, fv[:field].copy()), qs.value, ls.value

    def drain(self):
        """Run until every submitted request is finished; {id: (proof, queue_s, latency_s)}."""
        out = {}
        while True:
            pending = self.progress(wait=True)
            while True:
                r = self.take()
                if r is None:
                    break
                out[r[0]] = r[1:]
            if pending == 0 and not self._meta:
                return out

    def run_trace(self, kinds, num_vars, seeds, transcripts, arrival_s, field=FP3, proofs=True, host_tables=None):
        """Open-loop trace: request i arrives arrival_s[i] seconds after the
        start.  Tables from seeds[i] (generated on the device) or, with
        host_tables given, from host_tables[i] (one or two arrays of 2^n
        canonical words in host memory, uploaded on admission).  Returns
        (latency_s array, makespan_s, proofs or None) with the proofs
        concatenated as in Batch.prove_raw."""
        n = len(kinds)
        k = (ctypes.c_int * n)(*[int(x) for x in kinds])
        nv = (ctypes.c_uint32 * n)(*[int(x) for x in num_vars])
        tx = (vp * n)(*[t.h for t in transcripts])
        if host_tables is not None:
            keep = []
            ptrs = (u64p * (2 * n))()
            for i, tabs in enumerate(host_tables):
                for j, t in enumerate(tabs):
                    if isinstance(t, np.ndarray):
                        a = np.ascontiguousarray(t, dtype=np.uint64)
                        keep.append(a)
                        ptrs[2 * i + j] = _p(a)
                    else:   # a host address (e.g. a pinned torch tensor's data_ptr())
                        ptrs[2 * i + j] = ctypes.cast(ctypes.c_void_p(int(t)), u64p)
        arr = np.ascontiguousarray(np.asarray(arrival_s, dtype=np.float64))
        lat = np.zeros(n, dtype=np.float64)
        mk = ctypes.c_double()
        dpc = ctypes.POINTER(ctypes.c_double)
        rows = int(sum(int(x) for x in num_vars))
        rp = ch = fv = None
        if proofs:
            rp = np.zeros(rows * 2 * field, dtype=np.uint64)
            ch = np.zeros(rows * field, dtype=np.uint64)
            fv = np.zeros(n * field, dtype=np.uint64)
        outs = (_p(rp) if proofs else None, _p(ch) if proofs else None, _p(fv) if proofs else None)
        if host_tables is not None:
            check(load().effsc_server_run_trace_host(self.h, n, k, field, nv, ptrs, tx, arr.ctypes.data_as(dpc),
                                                     lat.ctypes.data_as(dpc), ctypes.byref(mk), *outs))
        else:
            sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))
            check(load().effsc_server_run_trace(self.h, n, k, field, nv, _p(sd), tx, arr.ctypes.data_as(dpc),
                                                lat.ctypes.data_as(dpc), ctypes.byref(mk), *outs))
        out = None
        if proofs:
            out = []
            ro = 0
            for i in range(n):
                d = 2 if int(kinds[i]) == IP else 1
                m = int(num_vars[i])
                rpi = rp[ro * 2 * field:(ro + m) * 2 * field].reshape(m, 2, field)[:, :d, :]
                out.append(SumcheckProof(rpi, ch[ro * field:(ro + m) * field].reshape(m, field),
                                         fv[i * field:(i + 1) * field]))
                ro += m
        return lat, mk.value, out


# ---------------------------------------------------------------------------
# streams (src/streams/)
# ---------------------------------------------------------------------------
def reorder_vec_msb(evaluations, ctx=None):
    """src/streams/memory/core.rs:20-47: out[i] = src[bit_reverse(i)]."""
    ctx = ctx or Context.default()
    a = np.ascontiguousarray(np.asarray(evaluations, dtype=np.uint64))
    ncomp = 3 if a.ndim == 2 else 1
    out = np.empty_like(a)
    check(load().effsc_reorder_msb(ctx.h, _p(a), a.shape[0], ncomp, _p(out)))
    return out


def multivariate_product_claim(streams, field=FP3, ctx=None):
    """src/streams/stream.rs:14-40: sum over the hypercube of the product."""
    ctx = ctx or Context.default()
    tabs = []
    for st in streams:
        t = st.evaluations if isinstance(st, (MemoryStream, FileStream)) else st
        tabs.append(np.asarray(t, dtype=np.uint64))
    if not tabs:
        raise AssertionError("should be given at least one stream")    # the reference asserts
    n = tabs[0].shape[0]
    if any(t.shape[0] != n for t in tabs):
        raise AssertionError("all streams should have the same number of variables")
    ncomp = 3 if any(t.ndim == 2 for t in tabs) else 1
    if ncomp == 3:
        tabs = [t if t.ndim == 2 else np.stack([t, np.zeros_like(t), np.zeros_like(t)], axis=1) for t in tabs]
    tabs = [t if t.flags["C_CONTIGUOUS"] else np.ascontiguousarray(t) for t in tabs]
    out = np.zeros(field, dtype=np.uint64)
    ptrs = (u64p * len(tabs))(*[t.ctypes.data_as(u64p) for t in tabs])
    check(load().effsc_stream_claim(ctx.h, field, len(tabs), ptrs, n, ncomp, _p(out)))
    return out


def multivariate_claim(stream, field=FP3, ctx=None):
    """src/streams/stream.rs:3-12: sum of a stream's evaluations."""
    return multivariate_product_claim([stream], field, ctx)


class MemoryStream:
    """src/streams/memory/core.rs:9-66: evaluations in MSB order."""

    def __init__(self, evaluations):
        e = np.asarray(evaluations, dtype=np.uint64)
        n = e.shape[0]
        if n == 0 or n & (n - 1):
            raise AssertionError("evaluations must be a non-empty power of two")
        self.evaluations = e

    @classmethod
    def new_from_lex_msb(cls, evaluations):
        return cls(reorder_vec_msb(evaluations))

    def evaluation(self, point):
        return self.evaluations[point]

    def num_variables(self):
        return int(self.evaluations.shape[0]).bit_length() - 1


class FileStream:
    """src/streams/file/core.rs: a file of base-field elements, 8
    little-endian canonical bytes each (arkworks' uncompressed encoding of a
    64-bit prime field element), memory-mapped; provers read it in place
    through from_host."""

    def __init__(self, path):
        self.path = path
        self.evaluations = np.memmap(path, dtype="<u8", mode="r")
        n = self.evaluations.shape[0]
        if n == 0 or n & (n - 1):
            raise AssertionError("file length must be a power of two elements")

    @staticmethod
    def write_to_file(path, data):
        np.asarray(data, dtype="<u8").tofile(path)

    @staticmethod
    def delete_file(path):
        import os
        os.remove(path)

    def evaluation(self, point):
        return self.evaluations[point]

    def num_variables(self):
        return int(self.evaluations.shape[0]).bit_length() - 1


def gen_uniform(seed, n, ctx=None):
    """Seeded uniform canonical table (host array)."""
    ctx = ctx or Context.default()
    out = np.empty(n, dtype=np.uint64)
    check(load().effsc_gen_uniform(ctx.h, seed, n, None, _p(out)))
    return out


def table_seed(seed, t):
    return int(load().effsc_table_seed(seed, t))


@dataclass
class ProductSumcheck:
    """Legacy return type, src/inner_product_sumcheck.rs:33-37."""
    prover_messages: list
    verifier_messages: list
    final_evaluations: tuple
    a: np.ndarray = None
    b: np.ndarray = None


@dataclass
class Sumcheck:
    """Legacy return type, src/multilinear_sumcheck.rs:31-35."""
    prover_messages: list
    verifier_messages: list
    final_evaluation: np.ndarray
    values: np.ndarray = None


def _rounds_for(n):
    return 0 if n == 0 else (n - 1).bit_length()


def inner_product_sumcheck_partial(a, b, transcript, num_rounds, hook=None, field=FP3):
    """src/inner_product_sumcheck.rs:507-565: sends (c0, c2) per round."""
    na = np.asarray(a).shape[0]
    if np.asarray(b).shape[0] != na:
        raise _lib.ReferencePanic(6, "a and b must have equal length")
    if num_rounds and (1 << _rounds_for(na)) < (1 << num_rounds):
        raise _lib.ReferencePanic(6, "num_rounds (%d) exceeds log2 of next-pow2 of len (%d)" % (num_rounds, na))
    pr = InnerProductProver(a, b, field=field)
    msgs, chals, prev = [], [], None
    for r in range(num_rounds):
        _, aux = pr.round(prev, aux=True)
        c0, c2 = aux[0], aux[1]
        msgs.append((c0, c2))
        transcript.send(c0)
        transcript.send(c2)
        if hook is not None:
            hook(r, transcript)
        prev = transcript.challenge()
        chals.append(prev)
    if prev is not None:
        pr.finalize(prev)
    ta, tb = pr.evaluations()
    fe = (ta[0], tb[0]) if len(ta) == 1 else (np.zeros(field, np.uint64), np.zeros(field, np.uint64))
    return ProductSumcheck(msgs, chals, fe, ta, tb)


def inner_product_sumcheck(a, b, transcript, hook=None, field=FP3):
    """src/inner_product_sumcheck.rs:568-585."""
    return inner_product_sumcheck_partial(a, b, transcript, _rounds_for(np.asarray(a).shape[0]), hook, field)


def multilinear_sumcheck_partial(values, transcript, num_rounds, hook=None, field=FP3):
    """src/multilinear_sumcheck.rs:265-319: sends (s0, s1) per round."""
    n = np.asarray(values).shape[0]
    if num_rounds and (1 << _rounds_for(n)) < (1 << num_rounds):
        raise _lib.ReferencePanic(6, "num_rounds (%d) exceeds log2 of next-pow2 of len (%d)" % (num_rounds, n))
    pr = MultilinearProver(values, field=field)
    msgs, chals, prev = [], [], None
    for r in range(num_rounds):
        _, aux = pr.round(prev, aux=True)
        msgs.append((aux[0], aux[1]))
        transcript.send(aux[0])
        transcript.send(aux[1])
        if hook is not None:
            hook(r, transcript)
        prev = transcript.challenge()
        chals.append(prev)
    if prev is not None:
        pr.finalize(prev)
    t = pr.evals()
    fe = t[0] if len(t) == 1 else np.zeros(field, np.uint64)
    return Sumcheck(msgs, chals, fe, t)


def multilinear_sumcheck(values, transcript, hook=None, field=FP3):
    """src/multilinear_sumcheck.rs:322-338."""
    return multilinear_sumcheck_partial(values, transcript, _rounds_for(np.asarray(values).shape[0]), hook, field)
