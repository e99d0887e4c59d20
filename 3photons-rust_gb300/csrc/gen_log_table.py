"""Generates tp_log_table.h: the table of the FP64 logarithm of the event
kernels (tp_math.h), computed with Python's arbitrary-precision decimal.

For j = 0..127, c_j = 1 + (j + 1/2)/128 is the centre of the j-th interval of
the mantissa m in [1, 2). r_j = 1/c_j rounded to 12 significant bits, so
that t = m r_j - 1 is small (|t| < 2^-8) and obtained with one FMA. The
table holds r_j and -log(r_j) split as hi + lo, hi a multiple of 2^-43 (so
that k ln2_hi + hi is exact) and lo the double nearest to the remainder.
Run: python gen_log_table.py > tp_log_table.h
"""
from decimal import Decimal, getcontext
import struct

getcontext().prec = 60


def round_bits(x, bits):
    """x (Decimal) rounded to `bits` significant bits, as a float."""
    f = float(x)
    m, e = __import__("math").frexp(f)
    scale = 2 ** bits
    return __import__("math").ldexp(round(m * scale) / scale, e)


def split(x, quantum_exp=43):
    q = Decimal(2) ** -quantum_exp
    hi = (x / q).to_integral_value() * q
    return float(hi), float(x - Decimal(float(hi)))


def main():
    ln2 = Decimal(2).ln()
    ln2_hi, ln2_lo = split(ln2, 42)  # k ln2_hi exact for |k| < 2^11
    print("// Generated by gen_log_table.py: table of tp_log (tp_math.h).")
    print("#ifndef TP_LOG_TABLE_H")
    print("#define TP_LOG_TABLE_H")
    print("#define TP_LN2_HI %r" % ln2_hi)
    print("#define TP_LN2_LO %r" % ln2_lo)
    print("// {r_j, -log(r_j) hi, -log(r_j) lo}, j = 0..127")
    print("#define TP_LOG_TABLE_INIT \\")
    print("  { \\")
    for j in range(128):
        c = Decimal(1) + (Decimal(j) + Decimal("0.5")) / 128
        r = round_bits(Decimal(1) / c, 12)
        L = -(Decimal(r).ln())
        hi, lo = split(L, 43)
        print("    {%r, %r, %r}, \\" % (r, hi, lo))
    print("  }")
    print("static const double kTpLogTable[128][3] = TP_LOG_TABLE_INIT;")
    print("#endif")


if __name__ == "__main__":
    main()
