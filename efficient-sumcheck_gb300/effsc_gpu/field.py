"""Small host-side field helpers for accessors (Goldilocks Fp and the crate's
F64Ext3 = Fp[X]/(X^3 - W), W = 7 * 2^-64 mod p, src/tests/fields.rs:73-100)."""
import numpy as np

P = 0xFFFFFFFF00000001
W = 0xFFFFFFF800000001
R = (1 << 64) % P
R_INV = pow(R, -1, P)


def to_canonical(x, repr=0):
    return int(x) % P if repr == 0 else int(x) * R_INV % P


def from_canonical(x, repr=0):
    return int(x) % P if repr == 0 else int(x) * R % P


def f_mul(a, b, field=3, repr=0):
    a = [to_canonical(x, repr) for x in np.asarray(a).reshape(-1)]
    b = [to_canonical(x, repr) for x in np.asarray(b).reshape(-1)]
    if field == 1:
        return np.array([from_canonical(a[0] * b[0] % P, repr)], dtype=np.uint64)
    prod = [0] * 5
    for i in range(3):
        for j in range(3):
            prod[i + j] += a[i] * b[j]
    c = [(prod[0] + W * prod[3]) % P, (prod[1] + W * prod[4]) % P, prod[2] % P]
    return np.array([from_canonical(x, repr) for x in c], dtype=np.uint64)


def _elem_list(a, field, repr):
    return [to_canonical(x, repr) for x in np.asarray(a).reshape(-1)[:field]]


def f_add(a, b, field=3, repr=0):
    x, y = _elem_list(a, field, repr), _elem_list(b, field, repr)
    return np.array([from_canonical((u + v) % P, repr) for u, v in zip(x, y)], dtype=np.uint64)


def f_sub(a, b, field=3, repr=0):
    x, y = _elem_list(a, field, repr), _elem_list(b, field, repr)
    return np.array([from_canonical((u - v) % P, repr) for u, v in zip(x, y)], dtype=np.uint64)


def f_scale(a, s, field=3, repr=0, inv=None):
    """a times the integer s, or times 1/inv."""
    m = pow(inv, -1, P) if inv is not None else s % P
    return np.array([from_canonical(u * m % P, repr) for u in _elem_list(a, field, repr)], dtype=np.uint64)
