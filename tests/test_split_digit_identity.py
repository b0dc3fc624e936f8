"""The integer identity behind the f64 split GEMM's slice digits (CPU only).

The split kernel takes each double x of a row with exponent e_r as the
fixed-point integer Y = x 2^(63 - e_r) (|Y| < 2^63) and cuts it into S
balanced base-128 digits without a per-digit rounding chain: with
C = 64 (2^49 + 2^42 + ... + 2^(56 - 7 (S-1))) + 2^(55 - 7 (S-1)),
lo = (Y mod 2^56) + C holds digit j + 64 (j >= 1) in bits [56 - 7j, 63 - 7j)
and its carry completes the top digit d_0 = (Y >> 56) + carry. This test
restates that arithmetic with exact integers and checks, over random,
subnormal and binade-edge values, that the sum never wraps, the digits stay
in [-128, 128] (top) and [-64, 63] (others), and the kept value equals a
digit-by-digit round-half-up recurrence: Y rounded to the nearest multiple of
2^(56 - 7 (S-1)), ties up.
"""

import random
import struct

M56 = (1 << 56) - 1


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _exp_above(b: int) -> int:
    """e with m < 2^e for the row maximum m given as |x| bits."""
    e = b >> 52
    if e:
        return e - 1022
    if b == 0:
        return 0
    return -1010 - (64 - b.bit_length())


def _fixed_point(x: float, e_r: int) -> int:
    u = _bits(x)
    e = (u >> 52) & 0x7FF
    mant = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
    sh = (e if e else 1) - 1012 - e_r
    y = (mant << min(sh, 63)) if sh >= 0 else ((mant >> -sh) if sh > -63 else 0)
    return -y if u >> 63 else y


def _carry_digits(y: int, s: int) -> list:
    c = 1 << (55 - 7 * (s - 1))
    for j in range(1, s):
        c += 64 << (56 - 7 * j)
    lo = (y & M56) + c
    assert lo < 1 << 57
    top = (y >> 56) + (lo >> 56)
    low = lo & M56
    return [top] + [((low >> (56 - 7 * j)) & 127) - 64 for j in range(1, s)]


def _recurrence_digits(y: int, s: int) -> list:
    out = []
    for j in range(s):
        k = 56 - 7 * j
        d = (y >> k) + ((y >> (k - 1)) & 1)
        y -= d << k
        out.append(d)
    return out


def _kept(ds: list) -> int:
    return sum(d << (56 - 7 * j) for j, d in enumerate(ds))


def test_carry_digits_equal_the_recurrence():
    rng = random.Random(2)
    for trial in range(4000):
        s = rng.randint(4, 8)
        scale = 2.0 ** rng.randint(-1000, 1000)
        row = [rng.choice([-1, 1]) * rng.random() ** rng.randint(1, 30) * scale for _ in range(8)]
        if trial % 7 == 0:
            row[0] = 2.0 ** rng.randint(-1070, -1023)  # subnormal
        if trial % 11 == 0:
            row = [(1 - 2 ** -53) * scale * rng.choice([-1, 1]) for _ in range(8)]  # top of a binade
        e_r = _exp_above(max(_bits(abs(v)) for v in row))
        k_last = 56 - 7 * (s - 1)
        for x in row:
            y = _fixed_point(x, e_r)
            assert abs(y) < 1 << 63
            ds = _carry_digits(y, s)
            assert -128 <= ds[0] <= 128
            assert all(-64 <= d <= 63 for d in ds[1:])
            q = (y + (1 << (k_last - 1))) >> k_last
            assert _kept(ds) == q << k_last
            assert _kept(ds) == _kept(_recurrence_digits(y, s))


def test_digit_to_bf16_is_exact():
    """0x4B400000 | f is the float 12582912 + f, so one FFMA gives (f - off) 2^-7s
    exactly, and a value with at most 8 significant bits is its float's upper half."""
    for f in range(257):
        v = struct.unpack("<f", struct.pack("<I", 0x4B400000 | f))[0]
        assert v == 12582912 + f
    for d in range(-128, 129):
        for s in range(8):
            val = struct.unpack("<f", struct.pack("<f", d * 2.0 ** (-7 * s)))[0]
            b = struct.unpack("<I", struct.pack("<f", val))[0]
            assert b & 0xFFFF == 0  # the bf16 (upper half) is exact
