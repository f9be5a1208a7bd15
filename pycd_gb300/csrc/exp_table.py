"""Print the constants of the KMC kernels' exp() (Tang's table-driven method,
ACM TOMS 15(2), 1989) for a table of 2^(j/256), as C source.

  x = (256 m + j) ln2/256 + r,  |r| <= ln2/512,
  exp(x) = 2^m * 2^(j/256) * (1 + expm1(r))

* kInvL = 256/ln2 rounded to double;
* kL1 = ln2/256 truncated to 34 significant bits, so that N * kL1 is exact
  for |N| < 2^19 (|x| < 745 gives |N| < 2.8e5); kL2 = ln2/256 - kL1 rounded;
* 2^(j/256) = hi + lo, hi = RN(2^(j/256)), lo = RN(2^(j/256) - hi); then
  |lo| < ulp(hi)/2, so hi + lo rounds to hi in double (checked below; the
  kernels rely on it).

Values come from 200-bit arithmetic (mpmath).  Run:
    python pycd_gb300/csrc/exp_table.py > /tmp/table.inc
"""
import struct

import mpmath as mp

mp.mp.prec = 200
TB = 256


def bits(x):
    return "0x%016xULL" % struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def main():
    ln2 = mp.log(2)
    L = ln2 / TB
    e = int(mp.floor(mp.log(L, 2)))
    q = mp.mpf(2) ** (e - 33)
    L1 = mp.floor(L / q) * q
    print("// kInvL = %r, kL1 = %r, kL2 = %r" % (float(TB / ln2), float(L1), float(L - L1)))
    hi = [mp.mpf(float(mp.mpf(2) ** (mp.mpf(j) / TB))) for j in range(TB)]
    lo = [mp.mpf(2) ** (mp.mpf(j) / TB) - h for j, h in enumerate(hi)]
    assert all(float(h) + float(l) == float(h) for h, l in zip(hi, lo))
    for name, vals in (("kExp2Hi", hi), ("kExp2Lo", lo)):
        print("static __device__ const unsigned long long %s[%d] = {" % (name, TB))
        for i in range(0, TB, 4):
            print("    " + ", ".join(bits(v) for v in vals[i:i + 4]) + ",")
        print("};")


if __name__ == "__main__":
    main()
