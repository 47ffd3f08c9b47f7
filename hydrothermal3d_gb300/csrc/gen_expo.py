"""Generates the constants of expo.h (exp and 10^x by Tang's table method).

Method: P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15(2):144-157, 1989.
x = (32 m + j) ln2/32 + r with |r| <= ln2/64; e^x = 2^m 2^(j/32) e^r, the 32
values 2^(j/32) stored as a double plus a correction, e^r by its Taylor
polynomial of degree 6 (truncation below 0.04 ulp on |r| <= ln2/64).  The
reduction constant ln2/32 (and log10(2)/32 for 10^x) is split Cody-Waite
style (W. J. Cody, W. Waite, "Software Manual for the Elementary Functions",
1980) into a head of 32 significant bits, whose product with any |N| < 2^16
is exact, and a rounded tail.

All values are computed here with Python's decimal module at 60 digits and
rounded once to double, so the table is reproducible on any machine:

    python hydrothermal3d_gb300/csrc/gen_expo.py > constants.txt

prints the block that expo.h holds between its BEGIN/END markers; a CPU test
regenerates it and compares.
"""
from decimal import Decimal, getcontext
import math

getcontext().prec = 60


def hexd(v: float) -> str:
    return float.hex(v)


def head(v: Decimal, bits: int) -> float:
    """v truncated to `bits` significant bits (exactly representable)."""
    e = math.frexp(float(v))[1]  # v = f 2^e, 0.5 <= f < 1
    return math.ldexp(int(v * Decimal(2) ** (bits - e)), e - bits)


def block() -> str:
    ln2 = Decimal(2).ln()
    ln10 = Decimal(10).ln()
    log10_2 = ln2 / ln10
    L = ln2 / 32
    L10 = log10_2 / 32
    L1 = head(L, 32)
    L2 = float(L - Decimal(L1))
    T1 = head(L10, 32)
    T2 = float(L10 - Decimal(T1))
    lines = ["// generated by gen_expo.py: do not edit",
             f"#define HT3D_EXPO_INV_L {hexd(float(32 / ln2))}  // 32/ln2",
             f"#define HT3D_EXPO_L1 {hexd(L1)}  // head of ln2/32 (32 bits)",
             f"#define HT3D_EXPO_L2 {hexd(L2)}  // ln2/32 - L1",
             f"#define HT3D_EXPO_INV_L10 {hexd(float(32 / log10_2))}  // 32 log2(10)",
             f"#define HT3D_EXPO_L10_1 {hexd(T1)}  // head of log10(2)/32 (32 bits)",
             f"#define HT3D_EXPO_L10_2 {hexd(T2)}  // log10(2)/32 - L10_1",
             f"#define HT3D_EXPO_LN10 {hexd(float(ln10))}  // ln 10"]
    fact = Decimal(1)
    for k in range(2, 7):
        fact *= k
        lines.append(f"#define HT3D_EXPO_A{k} {hexd(float(1 / fact))}  // 1/{k}!")
    hi, lo = [], []
    for j in range(32):
        s = (ln2 * j / 32).exp()
        h = float(s)
        hi.append(hexd(h))
        lo.append(hexd(float(s - Decimal(h))))
    lines.append("#define HT3D_EXPO_TABLE_HI \\")
    lines += [f"    {', '.join(hi[i:i + 4])}{',' if i + 4 < 32 else ''} \\" for i in range(0, 32, 4)]
    lines[-1] = lines[-1][:-2]
    lines.append("#define HT3D_EXPO_TABLE_LO \\")
    lines += [f"    {', '.join(lo[i:i + 4])}{',' if i + 4 < 32 else ''} \\" for i in range(0, 32, 4)]
    lines[-1] = lines[-1][:-2]
    return "\n".join(lines)


if __name__ == "__main__":
    print(block())
