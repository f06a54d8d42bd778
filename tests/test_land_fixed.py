"""The order-independent landings of the deterministic reverse products
(idwarp_gb300/csrc/idw_land.cuh: land_fixed, and k_land_convert in idw_api.cu)
restated word by word on the CPU: three 64-bit words, each landing's value in
two's complement with 2^E at bit 126, added word by word with the carry
computed from each word's old value as an atomic add returns it.  Any order of
the same landings gives the same 192-bit sum, and the converted double is
within a few ulp of the exact rational sum."""
import math
import random
from fractions import Fraction

import pytest

M64 = (1 << 64) - 1


def _words(v, E):
    """land_fixed's three words of v (2^E at bit 126)."""
    m, e = math.frexp(abs(v))  # |v| = m 2^e, 0.5 <= m < 1
    M = int(m * 2.0 ** 53)  # exact
    sh = min(e - 53 + 126 - E, 74)
    u0 = u1 = u2 = 0
    if sh >= 64:
        u1 = (M << (sh - 64)) & M64
    elif sh > 0:
        u0 = (M << sh) & M64
        u1 = M >> (64 - sh)
    elif sh > -64:
        u0 = M >> (-sh)
    if v < 0:
        u0 = (~u0 + 1) & M64
        c0 = 1 if u0 == 0 else 0
        u1 = (~u1 + c0) & M64
        c1 = 1 if (c0 and u1 == 0) else 0
        u2 = (~u2 + c1) & M64
    return u0, u1, u2


def _land(w, v, E):
    """One landing: three 64-bit atomic adds with the carries land_fixed forms."""
    if v == 0.0:
        return
    u0, u1, u2 = _words(v, E)
    o0 = w[0]
    w[0] = (o0 + u0) & M64
    k0 = 1 if (o0 + u0) & M64 < o0 else 0
    a1 = (u1 + k0) & M64
    k1a = 1 if a1 < u1 else 0
    o1 = w[1]
    w[1] = (o1 + a1) & M64
    k1 = (1 if (o1 + a1) & M64 < o1 else 0) + k1a
    a2 = (u2 + k1) & M64
    w[2] = (w[2] + a2) & M64


def _convert(w, E):
    """k_land_convert: sign, magnitude, and the three words as doubles."""
    u0, u1, u2 = w
    neg = (u2 >> 63) != 0
    if neg:
        u0 = (~u0 + 1) & M64
        c0 = 1 if u0 == 0 else 0
        u1 = (~u1 + c0) & M64
        c1 = 1 if (c0 and u1 == 0) else 0
        u2 = (~u2 + c1) & M64
    r = math.ldexp(float(u2), 2 + E) + math.ldexp(float(u1), E - 62) + math.ldexp(float(u0), E - 126)
    return -r if neg else r


def _sum(values, order):
    E = max(math.frexp(abs(v))[1] - 1 for v in values if v != 0.0)  # ilogb
    w = [0, 0, 0]
    for i in order:
        _land(w, values[i], E)
    return tuple(w), _convert(w, E)


@pytest.mark.parametrize("seed", range(6))
def test_order_independent_and_accurate(seed):
    rng = random.Random(seed)
    n = rng.choice([2, 17, 300])
    # mixed signs, magnitudes over 40 binades, and a cancelling pair
    values = [rng.choice([-1.0, 1.0]) * rng.random() * 2.0 ** rng.randint(-40, 0) for _ in range(n)]
    values += [0.75, -0.75]
    exact = sum(Fraction(v) for v in values)
    ref_words, ref = _sum(values, list(range(len(values))))
    for _ in range(5):
        order = list(range(len(values)))
        rng.shuffle(order)
        words, got = _sum(values, order)
        assert words == ref_words and got == ref
    scale = max(abs(v) for v in values)
    # truncation below 2^(E-126) per landing, then the conversion's roundings
    assert abs(Fraction(ref) - exact) <= Fraction(4 * len(values)) * Fraction(scale) * Fraction(2) ** -126 + \
        Fraction(abs(ref)) * Fraction(2) ** -51


def test_carries_across_words():
    # values whose words wrap: the carries must land in the next word
    values = [1.0 - 2.0 ** -53] * 5 + [-(1.0 - 2.0 ** -53)] * 3 + [2.0 ** -70] * 7
    words, got = _sum(values, list(range(len(values))))
    for perm in ([14, 0, 13, 1, 12, 2, 11, 3, 10, 4, 9, 5, 8, 6, 7], list(reversed(range(15)))):
        assert _sum(values, perm)[0] == words
    exact = sum(Fraction(v) for v in values)
    assert abs(Fraction(got) - exact) <= abs(exact) * Fraction(2) ** -50


def test_negative_total_and_zero():
    values = [-3.5, 1.25, -0.125, 2.375]  # sums to exactly 0
    words, got = _sum(values, [0, 1, 2, 3])
    assert words == (0, 0, 0) and got == 0.0
    values = [-3.5, 1.25]
    assert _sum(values, [1, 0])[1] == -2.25
