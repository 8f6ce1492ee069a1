"""Generates fft_consts.cuh: cos/sin(2 pi e / R) for the in-register DFT radices.

Run: python ad-dft_gb300/csrc/gen_fft_consts.py   (writes fft_consts.cuh beside it)
Entries that are exactly 0 or +-1 in exact arithmetic are written exactly.
"""
from pathlib import Path

import numpy as np

RADICES = (6, 8, 9, 10, 12, 15, 16)


def exact(x):
    for v in (0.0, 1.0, -1.0, 0.5, -0.5):
        if abs(x - v) < 1e-15:
            return v
    return x


def main():
    out = ["// Generated by gen_fft_consts.py: twiddles W_R^e = cos(2 pi e/R) - i sin(2 pi e/R).",
           "#pragma once", "namespace addft {", "template <int R> struct TwTab;"]
    for R in RADICES:
        c = [exact(np.cos(2 * np.pi * e / R)) for e in range(R)]
        s = [exact(np.sin(2 * np.pi * e / R)) for e in range(R)]
        out.append(f"template <> struct TwTab<{R}> {{")
        out.append("  static constexpr double c[" + str(R) + "] = {" + ", ".join(repr(float(x)) for x in c) + "};")
        out.append("  static constexpr double s[" + str(R) + "] = {" + ", ".join(repr(float(x)) for x in s) + "};")
        out.append("};")
    out.append("}  // namespace addft")
    Path(__file__).with_name("fft_consts.cuh").write_text("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
