"""Writes lp_math_tables.cuh: the constants of the float-float first stage of lp_math.cuh.

Every value is computed to 60 significant digits with Python's decimal module and split into a
binary32 pair hi + lo (hi the float nearest the value, lo the float nearest the remainder), so
each pair carries the value to about 2^-48 relative.

    kExp2Tab[j] = 2^(j/64),        j = 0..63     (Tang's table-driven exp)
    kAtanTab[j] = atan(j/128),     j = 0..128    (atan(t) = atan(c) + atan((t-c)/(1+tc)))
    kLn2By64    = ln2/64 split in three: a 10-bit head (exact products with |n| < 2^14), two tails
    kPi2, kPi   = pi/2 and pi as pairs

Run: python gen_math_tables.py  (rewrites lp_math_tables.cuh beside this script)
"""
import os
import struct
from decimal import Decimal, getcontext

getcontext().prec = 60


def f32(d):
    """Nearest binary32 to the Decimal d (through the nearest double, then a correction step)."""
    import numpy as np
    x = np.float32(float(d))
    # correct a possible double-rounding: compare the neighbours exactly
    best = x
    for cand in (np.nextafter(x, np.float32(-np.inf)), np.nextafter(x, np.float32(np.inf))):
        if abs(Decimal(float(cand)) - d) < abs(Decimal(float(best)) - d):
            best = cand
    return best


def hexf(x):
    import numpy as np
    v = float(np.float32(x))
    if v == 0.0:
        return "0.0f"
    return v.hex().replace("0x", "0x") + "f"


def split(d):
    hi = f32(d)
    lo = f32(d - Decimal(float(hi)))
    return hi, lo


def ln2():
    return Decimal(2).ln()


def atan(x):
    """atan for 0 <= x <= 1: two half-angle reductions, then the odd Taylor series."""
    x = Decimal(x)
    for _ in range(3):
        x = x / (1 + (1 + x * x).sqrt())
    s, term, k, x2 = Decimal(0), x, 0, x * x
    while True:
        t = term / (2 * k + 1)
        if abs(t) < Decimal(10) ** -58:
            break
        s += t if k % 2 == 0 else -t
        term *= x2
        k += 1
    return 8 * s


def pi():
    return 4 * atan(Decimal(1))


def main():
    import numpy as np
    out = []
    out.append("// lp_math_tables.cuh: generated by gen_math_tables.py (do not edit).")
    out.append("#pragma once")
    out.append("namespace lpm")
    out.append("{")
    out.append("__device__ const float2 kExp2Tab[64] = {")
    for j in range(64):
        hi, lo = split((Decimal(j) / 64 * ln2()).exp())
        out.append(f"    {{{hexf(hi)}, {hexf(lo)}}}, // 2^({j}/64)")
    out.append("};")
    out.append("__device__ const float2 kAtanTab[129] = {")
    for j in range(129):
        hi, lo = split(atan(Decimal(j) / 128))
        out.append(f"    {{{hexf(hi)}, {hexf(lo)}}}, // atan({j}/128)")
    out.append("};")
    L = ln2() / 64
    # head: L rounded to 10 significant bits
    e = 0
    v = L
    while v < 1:
        v *= 2
        e += 1
    head = Decimal(int((v * 512).to_integral_value())) / 512 / (Decimal(2) ** e)
    t1 = f32(L - head)
    t2 = f32(L - head - Decimal(float(t1)))
    assert float(np.float32(float(head))) == float(head)
    out.append(f"constexpr float kLn2By64Head = {hexf(np.float32(float(head)))};")
    out.append(f"constexpr float kLn2By64Mid = {hexf(t1)};")
    out.append(f"constexpr float kLn2By64Tail = {hexf(t2)};")
    hi, lo = split(pi() / 2)
    out.append(f"constexpr float kPi2FHi = {hexf(hi)};")
    out.append(f"constexpr float kPi2FLo = {hexf(lo)};")
    hi, lo = split(pi())
    out.append(f"constexpr float kPiFHi = {hexf(hi)};")
    out.append(f"constexpr float kPiFLo = {hexf(lo)};")
    out.append("} // namespace lpm")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lp_math_tables.cuh")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
