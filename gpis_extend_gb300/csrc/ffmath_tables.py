"""Generates the constant tables of ffmath.cuh (the float-float logarithm and sine /
cosine of the Box-Muller draws) from their definitions at 60 significant digits:
each value as a pair of floats (hi = the value rounded to float, lo = the rest
rounded to float), and the split constants of pi / 2, pi / 256 and ln 2.

    python gpis_extend_gb300/csrc/ffmath_tables.py > tables.txt
"""
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 60


def pi():
    # Machin: pi = 16 atan(1/5) - 4 atan(1/239)
    def atan_inv(n):
        x = Decimal(1) / n
        x2 = x * x
        s, t, k = Decimal(0), x, 0
        while True:
            term = t / (2 * k + 1)
            if abs(term) < Decimal(10) ** -58:
                break
            s += -term if k % 2 else term
            t *= x2
            k += 1
        return s
    return 16 * atan_inv(5) - 4 * atan_inv(239)


PI = pi()


def sin_cos(x):
    s, c, t, k = Decimal(0), Decimal(0), Decimal(1), 0
    while True:
        if k % 2 == 0:
            c += t if (k // 2) % 2 == 0 else -t
        else:
            s += t if (k // 2) % 2 == 0 else -t
        k += 1
        t = t * x / k
        if abs(t) < Decimal(10) ** -58:
            return s, c


def split(v, parts=2):
    out = []
    r = v
    for _ in range(parts):
        f = np.float32(float(r))
        out.append(f)
        r -= Decimal(float(f))
    return out


def c_float(f):
    f = np.float32(f)
    return "0.0f" if f == 0 else f"{float(f).hex()}f"


def main():
    print("// log(1 + j / 256), j = -64 .. 128")
    rows = []
    for j in range(-64, 129):
        v = (Decimal(256 + j) / 256).ln()
        h, l = split(v)
        rows.append(f"    {{{c_float(h)}, {c_float(l)}}},")
    print("\n".join(rows))
    print("// sin and cos of j pi / 1024, j = 0 .. 256")
    rows = []
    for j in range(0, 257):
        s, c = sin_cos(PI * j / 1024)
        sh, sl = split(s)
        ch, cl = split(c)
        rows.append(f"    {{{c_float(sh)}, {c_float(sl)}, {c_float(ch)}, {c_float(cl)}}},")
    print("\n".join(rows))
    print("// pi / 2 in four parts, pi / 1024 in three, ln 2 in two")
    print(", ".join(c_float(x) for x in split(PI / 2, 4)))
    print(", ".join(c_float(x) for x in split(PI / 1024, 3)))
    print(", ".join(c_float(x) for x in split(Decimal(2).ln(), 2)))


if __name__ == "__main__":
    main()
