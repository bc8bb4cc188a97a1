"""The fixed-point cosine and sine (fixed_cos.cuh: turns_of, cos_turns_q62, sincos_turns_q62,
prob_q63, turns_q64_host) restated step for step in Python integers, against exact values from
cos_table.py's 256-bit arithmetic, and the committed constant file against its generator. The GPU's
own results are checked against the same exact values in test_gpu_field.py (internal-field walk) and
through the general-direction PFGSE parity tests."""
import math
import os
import random
import struct
import sys
from fractions import Fraction

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "randomwalk_nmr_gb300", "csrc")
sys.path.insert(0, CSRC)
import cos_table  # noqa: E402

C = cos_table.constants()
M64 = (1 << 64) - 1
M32 = (1 << 32) - 1
BOUND_Q62 = 2.5  # |cos_q62(x) - cos(x) * 2^62| < 2.5


def umulhi(a, b):
    return (a * b) >> 64


def umulhi32(a, b):
    return (a * b) >> 32


def turns_of(phase):
    """fixed_cos.cuh turns_of: (theta, g) or None where the kernels fall back to CUDA's cos."""
    bits = struct.unpack("<Q", struct.pack("<d", phase))[0]
    ex = (bits >> 52) & 0x7FF
    if ex >= 1063:
        return None
    sh = 1139 - ex
    theta = g = 0
    if ex != 0 and sh < 178:
        m = (bits & ((1 << 52) - 1)) | (1 << 52)
        lo2 = (m * C["INV_2PI_HI"]) & M64
        q1 = (umulhi(m, C["INV_2PI_LO"]) + lo2) & M64
        q2 = (umulhi(m, C["INV_2PI_HI"]) + (1 if q1 < lo2 else 0)) & M64
        theta = ((q1 >> (sh - 64)) | (q2 << (128 - sh))) & M64 if sh < 128 else q2 >> (sh - 128)
        g = ((q1 >> (sh - 66)) if sh < 130 else (q2 >> (sh - 130))) & 3
    return theta, g


def turn_parts(theta, g):
    """fixed_cos.cuh turn_parts: (C, S, dev, sr, quadrant, neg_r)."""
    tr = (theta + (1 << 51)) & M64
    k = tr >> 52
    d = (theta - (tr & ~((1 << 52) - 1))) & M64
    d = (d - (1 << 64) if d >> 63 else d) * 4 + g
    neg_r = d < 0
    a = -d if neg_r else d
    R = umulhi((a << 10) & M64, C["TWO_PI_Q61"])
    u = umulhi(R, R)
    u32, r32 = (u >> 31) & M32, (R >> 31) & M32
    hi3 = umulhi32(r32, u32)
    dev = (u >> 20) - umulhi32(umulhi32(u32, u32), C["C_INV3072"])
    sr = R - ((hi3 * C["C_INV6"]) >> 20) + umulhi32(umulhi32(hi3, u32), C["C_INV15360"])
    cj, sj = C["table"][k & (cos_table.QUADRANT - 1)]
    return cj, sj, dev, sr, (k >> 10) & 3, neg_r


def mul_cos_r(A, dev):
    return (A >> 1) - umulhi(A, dev)


def mul_sin_r(A, sr):
    return (umulhi(A, sr) + 512) >> 10


def cos_turns_q62(theta, g=0):
    cj, sj, dev, sr, q, neg_r = turn_parts(theta, g)
    odd = q & 1
    p1 = mul_cos_r(sj if odd else cj, dev)
    p2 = mul_sin_r(cj if odd else sj, sr)
    v = p1 - p2 if bool(odd) == neg_r else p1 + p2
    return -v if (q + 1) & 2 else v


def sincos_turns_q62(theta, g=0):
    cj, sj, dev, sr, q, neg_r = turn_parts(theta, g)
    cc, sc = mul_cos_r(cj, dev), mul_cos_r(sj, dev)
    cs, ss = mul_sin_r(cj, sr), mul_sin_r(sj, sr)
    cphi = cc + ss if neg_r else cc - ss
    sphi = sc - cs if neg_r else sc + cs
    odd, high = bool(q & 1), bool(q & 2)
    c0, s0 = (sphi, cphi) if odd else (cphi, sphi)
    return (-c0 if odd != high else c0), (-s0 if high else s0)


def cos_q62(phase):
    """fixed_cos.cuh cos_q62; None where the kernels fall back to CUDA's cos."""
    t = turns_of(phase)
    return None if t is None else cos_turns_q62(*t)


def turns_q64_host(x):
    """fixed_cos.cuh turns_q64_host."""
    ax = abs(x)
    bits = struct.unpack("<Q", struct.pack("<d", ax))[0]
    ex = bits >> 52
    if ex == 0 or ex >= 1063:
        return 0
    s = 1139 - ex - 66
    if s >= 128:
        return 0
    m = (bits & ((1 << 52) - 1)) | (1 << 52)
    W = ((m * C["INV_2PI_LO"]) >> 64) + m * C["INV_2PI_HI"]
    t66 = (W >> s) & ((1 << 66) - 1)
    theta = ((t66 + 2) >> 2) & M64
    return (-theta) & M64 if x < 0 else theta


def prob_q63(p):
    """field_kernels.cu prob_q63."""
    bits = struct.unpack("<Q", struct.pack("<d", p))[0]
    ex = (bits >> 52) & 0x7FF
    if ex < 959:
        return 0
    m = (bits & ((1 << 52) - 1)) | (1 << 52)
    sh = ex - 1012
    if sh >= 0:
        return m << sh
    r = -sh
    q, rem, half = m >> r, m & ((1 << r) - 1), 1 << (r - 1)
    return q + (1 if rem > half or (rem == half and q & 1) else 0)


def exact_cos_q62(phase):
    """cos(phase) * 2^62 as an exact fraction (256-bit reduction and series)."""
    fr = Fraction(phase)
    x = (abs(fr.numerator) << cos_table.BITS) // fr.denominator
    x %= 2 * cos_table.PI
    half_pi = cos_table.PI // 2
    q = x // half_pi
    c, s = cos_table.cos_sin(x - q * half_pi)
    return Fraction([c, -s, -c, s][q % 4] << 62, 1 << cos_table.BITS)


def exact_sincos_turns_q62(t):
    """(cos, sin)(2 pi t) * 2^62 as exact fractions, t a Fraction of a turn."""
    t = t - (t.numerator // t.denominator)
    q4 = t * 4
    q = q4.numerator // q4.denominator
    c, s = cos_table.cos_sin(int((q4 - q) * (cos_table.PI // 2)))  # the angle within its quadrant
    cv, sv = [(c, s), (-s, c), (-c, -s), (s, -c)][q % 4]
    return Fraction(cv << 62, 1 << cos_table.BITS), Fraction(sv << 62, 1 << cos_table.BITS)


def test_constant_file_matches_generator():
    with open(os.path.join(CSRC, "cos_table.inc")) as f:
        assert f.read() == cos_table.render()


def test_generator_constants():
    assert abs(cos_table.PI / 2 ** cos_table.BITS - math.pi) < 1e-15
    assert abs(C["TWO_PI_Q61"] / 2.0 ** 61 - 2 * math.pi) < 1e-15
    assert abs(((C["INV_2PI_HI"] << 64) | C["INV_2PI_LO"]) / 2.0 ** 128 - 1 / (2 * math.pi)) < 1e-17
    for j, (cv, sv) in enumerate(C["table"]):
        assert abs(cv / 2.0 ** 63 - math.cos(j * math.pi / 2048)) < 1e-15
        assert abs(sv / 2.0 ** 63 - math.sin(j * math.pi / 2048)) < 1e-15
    assert len(C["table"]) == cos_table.QUADRANT == 1024
    assert C["table"][0] == (1 << 63, 0)


def phases(n, seed):
    rng = random.Random(seed)
    out = [0.0, -0.0, 5e-324, 1e-300, 1e-20, 2.0 ** -62, 1.0, -1.0, math.pi, math.pi / 2, -math.pi / 2,
           2.0 ** 40 - 1.0, -(2.0 ** 40 - 1.0), 1e6, 12345.678]
    for _ in range(n):
        r = rng.random()
        if r < 0.3:
            out.append(rng.uniform(-10.0, 10.0))
        elif r < 0.6:
            out.append(rng.uniform(-1e4, 1e4))
        elif r < 0.8:
            out.append(rng.uniform(-1e11, 1e11))
        else:  # at the table's and the quadrants' boundaries
            out.append(rng.randint(-400000, 400000) * math.pi / 2048 + rng.uniform(-1e-12, 1e-12))
    return out


def test_fixed_point_cosine_error_bound():
    worst = Fraction(0)
    for x in phases(6000, 11):
        err = abs(cos_q62(x) - exact_cos_q62(x))
        worst = max(worst, err)
    assert worst < BOUND_Q62, float(worst)


def test_fixed_point_cosine_declines_large_and_nonfinite_phases():
    for x in (2.0 ** 40, -(2.0 ** 41), 1e300, math.inf, -math.inf, math.nan):
        assert cos_q62(x) is None
    assert cos_q62(0.0) == 1 << 62 and cos_q62(5e-324) == 1 << 62


def test_probability_conversion_rounds_like_the_tables():
    rng = np.random.default_rng(2)
    vals = [0.0, 1.0, 0.5, 2.0 ** -64, 2.0 ** -63, 3 * 2.0 ** -65, 5e-324, np.nextafter(1.0, 0.0)]
    f = rng.uniform(0.9, 1.0, 50)
    for fv in f:  # repeated products, as the walk builds them
        v = 1.0
        for _ in range(int(rng.integers(1, 3000))):
            v = v * fv
        vals.append(v)
    vals += list(rng.uniform(0.0, 1.0, 200)) + list(2.0 ** rng.uniform(-70, 0, 200))
    for v in vals:
        assert prob_q63(float(v)) == round(Fraction(float(v)) * 2 ** 63), v  # round half to even


@pytest.mark.parametrize("seed", [1, 2])
def test_echo_term_error_bound(seed):
    """E * 2^61 from pAlive * 2^63 and cos * 2^62 (field_kernels.cu echo_term): below 3 units."""
    rng = random.Random(seed)
    for x in phases(500, seed):
        pal = rng.choice([1 << 63, 0, rng.randrange(1 << 63)])
        c62 = cos_q62(x)
        m = umulhi(pal, abs(c62))
        e = -m if c62 < 0 else m
        assert abs(e - Fraction(pal, 1 << 63) * exact_cos_q62(x) / 2) < 3


def test_sincos_in_turns_error_bound():
    rng = random.Random(21)
    thetas = [0, 1, (1 << 64) - 1, 1 << 62, 1 << 63, 3 << 62, 1 << 52, (1 << 52) - 1, 1 << 51, (1 << 51) + 1]
    thetas += [k << 52 for k in range(0, 4096, 97)] + [(k << 52) + rng.randint(-3, 3) for k in range(0, 4096, 131)]
    thetas += [rng.getrandbits(64) for _ in range(4000)]
    worst = Fraction(0)
    for th in thetas:
        th &= M64
        for g in (0, 3):
            c, s_ = sincos_turns_q62(th, g)
            assert c == cos_turns_q62(th, g)
            ec, es = exact_sincos_turns_q62(Fraction(th * 4 + g, 1 << 66))
            worst = max(worst, abs(c - ec), abs(s_ - es))
    assert worst < BOUND_Q62, float(worst)


def test_host_turns_exact_to_a_unit():
    """turns_q64_host(x) within one unit of 2^64 frac(x / (2 pi)), for both signs."""
    rng = random.Random(8)
    xs = [1.0, -1.0, math.pi, 2 * math.pi, 1e-3, -1e-3, 0.1234, 5e-20, 1e6 + 0.5, -(2.0 ** 39)]
    xs += [rng.uniform(-1e4, 1e4) for _ in range(500)] + [rng.uniform(-1e-6, 1e-6) for _ in range(100)]
    two_pi = Fraction(2 * cos_table.PI, 1 << cos_table.BITS)
    for x in xs:
        t = Fraction(x) / two_pi
        t -= t.numerator // t.denominator
        exact = t * (1 << 64)
        got = turns_q64_host(x)
        diff = abs(got - exact)
        diff = min(diff, abs(diff - (1 << 64)))  # the turn wraps
        assert diff <= 1, (x, float(diff))
    assert turns_q64_host(0.0) == 0 and turns_q64_host(2.0 ** 41) == 0
