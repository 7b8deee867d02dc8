"""Big-integer restatement of the coefficient provers with a RoundPolyEvaluator
callback and tablewise tables, for the declarative-evaluator tests.

Follows src/provers/coefficient.rs (MSB: pairs (k, k + L/2), msb_fold_vec and
msb_fold_tablewise :131-160, the EvalsInfty wire :272-294, final_value
:300-329), src/provers/coefficient_lsb.rs (pairs (2k, 2k+1), reduce :137-166,
final_value :215-236) and the legacy runner coefficient_sumcheck
(src/coefficient_sumcheck.rs:255-365).  The four evaluators are the
reference's own test evaluators (src/coefficient_sumcheck.rs:379-430),
restated as callbacks (the form the crate takes) next to their declarative
form (effsc_gpu.Evaluator, the form the device takes)."""
import bigint_ref as R

P = R.P
INV2 = (P + 1) // 2


def _fe(x):
    return R.lift(x) if isinstance(x, int) else tuple(int(v) % P for v in x)


# ---- the reference's test evaluators as callbacks (coeffs, tw pairs, pw pairs)
def degree1(coeffs, tw, pw):
    even, odd = pw[0]
    coeffs[0] = R.add(coeffs[0], even)
    coeffs[1] = R.add(coeffs[1], R.sub(odd, even))


def degree2(coeffs, tw, pw):
    s0, s1 = pw[0]
    s2 = R.add(s0, s1)
    c1 = R.mul(R.add(R.sub(R.mul(R.lift(P - 3), s0), s2), R.mul(R.lift(4), s1)), R.lift(INV2))
    c2 = R.mul(R.add(R.sub(s0, R.mul(R.lift(2), s1)), s2), R.lift(INV2))
    coeffs[0] = R.add(coeffs[0], s0)
    coeffs[1] = R.add(coeffs[1], c1)
    coeffs[2] = R.add(coeffs[2], c2)


def mixed(coeffs, tw, pw):
    coeffs[0] = R.add(coeffs[0], R.add(tw[0][0][0], pw[0][0]))


def inner_product(coeffs, tw, pw):
    (ae, ao), (be, bo) = pw[0], pw[1]
    coeffs[0] = R.add(coeffs[0], R.mul(ae, be))
    coeffs[1] = R.add(coeffs[1], R.sub(R.mul(ao, bo), R.mul(ae, be)))


EVALUATORS = {"degree1": (degree1, 1), "degree2": (degree2, 2), "mixed": (mixed, 0),
              "inner_product": (inner_product, 1)}


def declarative(E, name):
    """The same evaluators as sums of constant multiples of products of pair
    elements (Degree2's coefficients expanded: s2 = s0 + s1 gives
    c1 = (-4 s0 + 3 s1) / 2 = -2 s0 + (3/2) s1, c2 = (2 s0 - s1) / 2 = s0 - s1 / 2)."""
    m1 = P - 1
    if name == "degree1":
        return E.Evaluator(1, [(0, 1, [E.pw_even(0)]), (1, 1, [E.pw_odd(0)]), (1, m1, [E.pw_even(0)])])
    if name == "degree2":
        return E.Evaluator(2, [(0, 1, [E.pw_even(0)]), (1, P - 2, [E.pw_even(0)]), (1, 3 * INV2 % P, [E.pw_odd(0)]),
                               (2, 1, [E.pw_even(0)]), (2, P - INV2, [E.pw_odd(0)])])
    if name == "mixed":
        return E.Evaluator(0, [(0, 1, [E.tw_even(0, 0)]), (0, 1, [E.pw_even(0)])])
    if name == "inner_product":
        return E.Evaluator(1, [(0, 1, [E.pw_even(0), E.pw_even(1)]), (1, 1, [E.pw_odd(0), E.pw_odd(1)]),
                               (1, m1, [E.pw_even(0), E.pw_even(1)])])
    raise KeyError(name)


def horner(c, x):
    r = R.ZERO
    for v in reversed(c):
        r = R.add(R.mul(r, x), v)
    return r


class RefPanic(Exception):
    """Where the reference panics."""


class RefCoefProver:
    """CoefficientProver / CoefficientProverLSB with a callback evaluator."""

    def __init__(self, order, evaluate, degree, tablewise, pairwise):
        self.order, self.evaluate, self.deg = order, evaluate, degree
        self.tw = [[[_fe(x) for x in row] for row in t] for t in tablewise]
        self.pw = [[_fe(x) for x in t] for t in pairwise]

    def _n(self):
        return len(self.tw[0]) if self.tw else (len(self.pw[0]) if self.pw else 0)

    def coefficients(self):
        n = self._n()
        half = n // 2
        coeffs = [R.ZERO] * (self.deg + 1)
        for k in range(half):
            lo, hi = (k, k + half) if self.order == "msb" else (2 * k, 2 * k + 1)
            tw = [(t[lo], t[hi]) for t in self.tw]
            pw = [(t[lo], t[hi]) for t in self.pw]
            self.evaluate(coeffs, tw, pw)
        return coeffs

    def reduce(self, c):
        def fold_pair(a, b):
            return R.add(a, R.mul(c, R.sub(b, a)))
        n = self._n()
        half = n // 2
        if self.order == "msb":
            if n > 1:
                self.pw = [[fold_pair(t[k], t[k + half]) for k in range(half)] for t in self.pw]
                self.tw = [[[fold_pair(x, y) for x, y in zip(t[k], t[k + half])] for k in range(half)] for t in self.tw]
        else:
            self.pw = [[fold_pair(t[2 * k], t[2 * k + 1]) for k in range(len(t) // 2)] for t in self.pw]
            self.tw = [[[fold_pair(x, y) for x, y in zip(t[2 * k], t[2 * k + 1])] for k in range(len(t) // 2)]
                       for t in self.tw]

    def round(self, c=None):
        if c is not None:
            self.reduce(c)
        coeffs = self.coefficients()
        d = self.deg
        if d <= 1:
            return [coeffs[0]], coeffs
        return [coeffs[0], coeffs[d]] + [horner(coeffs, R.lift(i)) for i in range(2, d)], coeffs

    def finalize(self, c):
        self.reduce(c)

    def final_value(self):
        lone = len(self.pw) == 1 and not self.tw and len(self.pw[0]) == 1
        if lone and (self.order == "msb" or self.deg == 1):
            return self.pw[0][0]
        coeffs = [R.ZERO] * (self.deg + 1)
        tw = [(t[0], None) if len(t) == 1 else (None, None) for t in self.tw]
        pw = [(t[0], R.ZERO) if len(t) == 1 else (R.ZERO, R.ZERO) for t in self.pw]
        try:
            self.evaluate(coeffs, tw, pw)
        except TypeError:
            # the reference indexes an empty slice here and panics
            raise RefPanic("final_value reads an empty tablewise row")
        return R.add(horner(coeffs, R.ZERO), horner(coeffs, R.ONE))
