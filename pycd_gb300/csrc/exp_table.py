"""Print exp_seed.h: the constants of the KMC kernels' exp() (Tang's
table-driven method, ACM TOMS 15(2), 1989, with a table of 2^(j/4096)) and
the two seed tables the library builds that table from.

  x = (4096 m + j) ln2/4096 + r,  |r| <= ln2/8192,
  exp(x) = 2^m * 2^(j/4096) * (1 + expm1(r))

* kInvL = 4096/ln2 rounded to double;
* kL1 = ln2/4096 truncated to 30 significant bits, so that N * kL1 is exact
  for |N| < 2^23 (|x| < 745 gives |N| < 4.5e6); kL2 = ln2/4096 - kL1 rounded;
* seeds: 2^(a/256) (a < 256) and 2^(b/4096) (b < 16), each as hi + lo with
  hi = RN(value), lo = RN(value - hi); |lo| < ulp(hi)/2, so hi + lo rounds
  to hi in double (checked below).  The library forms 2^((16 a + b)/4096)
  as a double-double product of the two (exact FMA arithmetic, the same on
  every host) and keeps it as hi + lo.

Values come from 200-bit arithmetic (mpmath).  Run:
    python pycd_gb300/csrc/exp_table.py > pycd_gb300/csrc/exp_seed.h
"""
import struct

import mpmath as mp

mp.mp.prec = 200
TB = 4096


def bits(x):
    return "0x%016xULL" % struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def seed(n, den):
    hi = [mp.mpf(float(mp.mpf(2) ** (mp.mpf(j) / den))) for j in range(n)]
    lo = [mp.mpf(2) ** (mp.mpf(j) / den) - h for j, h in enumerate(hi)]
    assert all(float(h) + float(l) == float(h) for h, l in zip(hi, lo))
    return hi, lo


def table(name, vals):
    out = ["static const unsigned long long %s[%d] = {" % (name, len(vals))]
    for i in range(0, len(vals), 4):
        out.append("    " + ", ".join(bits(v) for v in vals[i:i + 4]) + ",")
    out.append("};")
    return out


def main():
    ln2 = mp.log(2)
    L = ln2 / TB
    e = int(mp.floor(mp.log(L, 2)))
    q = mp.mpf(2) ** (e - 29)
    L1 = mp.floor(L / q) * q
    lines = [
        "// Constants and seed tables of the KMC kernels' exp(); printed by",
        "// exp_table.py (200-bit arithmetic).",
        "#pragma once",
        "",
        "// 4096/ln2, and ln2/4096 = PYCD_EXP_L1 + PYCD_EXP_L2 (L1 to 30 bits)",
        "#define PYCD_EXP_INVL %r" % float(TB / ln2),
        "#define PYCD_EXP_L1 %r" % float(L1),
        "#define PYCD_EXP_L2 %r" % float(L - L1),
        "",
        "// 2^(a/256) = kExpSeedHi256[a] + kExpSeedLo256[a]",
    ]
    hi, lo = seed(256, 256)
    lines += table("kExpSeedHi256", hi) + table("kExpSeedLo256", lo)
    lines += ["", "// 2^(b/4096) = kExpSeedHi16[b] + kExpSeedLo16[b]"]
    hi, lo = seed(16, TB)
    lines += table("kExpSeedHi16", hi) + table("kExpSeedLo16", lo)
    print("\n".join(lines))


if __name__ == "__main__":
    main()
