"""Writes cos_table.inc: the constants of the fixed-point cosine (fixed_cos.cuh).

Every value is computed in exact integer arithmetic: pi from Machin's formula
pi = 16 atan(1/5) - 4 atan(1/239), sines and cosines from their Taylor series, all in fixed point
with 256 fraction bits, then rounded to nearest. Run `python cos_table.py` to regenerate; the test
suite checks that the committed file matches this script's output.
"""
import os

BITS = 256
ONE = 1 << BITS


def atan_inv(n):
    """atan(1/n) * 2^BITS by its Taylor series."""
    total, term, k, sign = 0, ONE // n, 1, 1
    n2 = n * n
    while term:
        total += sign * (term // k)
        term //= n2
        k += 2
        sign = -sign
    return total


PI = 16 * atan_inv(5) - 4 * atan_inv(239)


def cos_sin(x):
    """(cos x, sin x) * 2^BITS for x * 2^BITS given, |x| <= pi / 2."""
    c, s = ONE, x
    term_c, term_s, n = ONE, x, 1
    while term_c or term_s:
        term_c = -term_c * x // ONE * x // ONE // ((2 * n - 1) * (2 * n))
        term_s = -term_s * x // ONE * x // ONE // ((2 * n) * (2 * n + 1))
        c += term_c
        s += term_s
        n += 1
    return c, s


def rnd(num, den):
    """num / den rounded to nearest (num, den > 0)."""
    return (2 * num + den) // (2 * den)


QUADRANT = 1024  # table entries per quadrant: |r| <= pi / 4096 after the reduction


def constants():
    table = []
    for j in range(QUADRANT):  # j * pi / 2048: the first quadrant in 1/4096-turn steps
        c, s = cos_sin(PI * j // (2 * QUADRANT))
        table.append((rnd(c << 63, ONE), rnd(s << 63, ONE)))
    two_pi = 2 * PI
    k = rnd(ONE << 128, two_pi)  # 2^128 / (2 pi)
    return dict(
        table=table,
        INV_2PI_HI=k >> 64,
        INV_2PI_LO=k & ((1 << 64) - 1),
        TWO_PI_Q61=rnd(two_pi << 61, ONE),
        C_INV6=rnd(1 << 32, 6),
        C_INV3072=rnd(1 << 32, 3072),
        C_INV15360=rnd(1 << 32, 15360),
    )


def render():
    c = constants()
    lines = ["// Generated by cos_table.py (exact integer arithmetic); do not edit.",
             "// Fixed-point cosine of the field walk: 2^128 / (2 pi) in two words, 2 pi * 2^61, the 32-bit",
             "// reciprocals 2^32 / 6, / 3072, / 15360 of the Taylor terms, and cos / sin (j pi / 2048) * 2^63",
             f"// for j = 0 .. {QUADRANT - 1}."]
    for name in ("INV_2PI_HI", "INV_2PI_LO", "TWO_PI_Q61"):
        lines.append(f"constexpr uint64_t {name} = 0x{c[name]:016x}ull;")
    for name in ("C_INV6", "C_INV3072", "C_INV15360"):
        lines.append(f"constexpr uint32_t {name} = {c[name]}u;")
    lines.append(f"constexpr int kQuadrant = {QUADRANT};")
    lines.append(f"__device__ const uint64_t kQuadrantCosSin[{QUADRANT}][2] = {{")
    for cv, sv in c["table"]:
        lines.append(f"    {{0x{cv:016x}ull, 0x{sv:016x}ull}},")
    lines.append("};")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cos_table.inc")
    with open(out, "w") as f:
        f.write(render())
