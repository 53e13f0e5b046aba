"""Numbers of SVG path data are rounded as Rust's f32::from_str rounds them (the nearest f32, ties
to even, from the exact decimal value), which lyon's parser calls (crates/extra/src/parser.rs:
413-467). The library's parser (host threads) must give the bits the exact rational rounding of
the oracle gives, including the cases a conversion through f64 gets wrong: values within a hair
of a midpoint between two floats, exact midpoints, subnormals, overflow, and more digits than
any float needs."""

import struct
from fractions import Fraction

import numpy as np

from lyon_gb300 import svg
from oracle.svg_oracle import decimal_to_f32


def _exact_decimal(fr: Fraction) -> str:
    """The exact decimal expansion of a dyadic rational (terminates)."""
    neg = fr < 0
    fr = abs(fr)
    digits = 0
    while (fr * 10 ** digits).denominator != 1:
        digits += 1
    n = int(fr * 10 ** digits)
    s = str(n).rjust(digits + 1, "0")
    out = s[:-digits] + "." + s[-digits:] if digits else s
    return ("-" if neg else "") + out


def _f32(bits: int) -> float:
    return struct.unpack("<f", struct.pack("<I", bits))[0]


def _cases(seed=3):
    rng = np.random.default_rng(seed)
    out = []
    # Midpoints between neighbouring floats, exactly and a hair either side, across the range.
    for _ in range(300):
        bits = int(rng.integers(1, 0x7F7FFFFF))
        lo = Fraction(_f32(bits))
        hi = Fraction(_f32(bits + 1))
        mid = (lo + hi) / 2
        d = _exact_decimal(mid)
        out.append(d)
        out.append(d + "000000000000000000001")
        # just below: subtract one in the last place
        digits = len(d.split(".")[1]) if "." in d else 0
        below = mid - Fraction(1, 10 ** (digits + 3))
        out.append(_exact_decimal(below))
    # Random decimals with 1..40 significant digits and exponents across the float range.
    for _ in range(400):
        nd = int(rng.integers(1, 41))
        digits = "".join(str(int(x)) for x in rng.integers(0, 10, nd)).lstrip("0") or "1"
        e = int(rng.integers(-60, 45))
        sign = "-" if rng.random() < 0.3 else ""
        point = int(rng.integers(0, len(digits) + 1))
        mant = digits[:point] + "." + digits[point:] if point < len(digits) else digits
        if mant.startswith("."):
            mant = "0" + mant
        out.append(f"{sign}{mant}e{e}")
    # Subnormals, the edges of the range, zeros, long strings.
    out += ["1e-45", "7e-46", "7.006492321624085e-46", "7.006492321624086e-46", "1.17549435e-38",
            "1.1754942e-38", "3.4028235e38", "3.4028236e38", "3.40282356779733661637539395458142568448e38",
            "3.40282356779733661637539395458142568447e38", "1e39", "0", "-0", "0.000", "00012.5000",
            "1" + "0" * 60, "0." + "0" * 50 + "1", "9" * 150, "1." + "0" * 130 + "1",
            "0.1", "0.2", "0.3", "16777217", "16777216.5", "33554435", "1e10", "1e11", "1e22",
            "1e23", "123456789e-10", "5e-324", "2.5e-45"]
    return out


def test_library_parser_rounds_numbers_exactly():
    nums = _cases()
    strings = [f"M {x} 1" for x in nums]
    parsed = svg.parse_paths(strings)
    assert (parsed.status == 0).all()
    pts = parsed.batch.points
    po = parsed.batch.point_offsets
    bad = []
    for i, x in enumerate(nums):
        got = np.float32(pts[po[i]][0])
        want = decimal_to_f32(x)
        if got.tobytes() != want.tobytes():
            bad.append((x, got, want))
    assert not bad, bad[:5]
