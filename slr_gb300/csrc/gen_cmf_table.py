#!/usr/bin/env python3
"""Generates ``cmf_table.inc``: the CIE 1931 2-degree colour matching
functions at 1 nm steps over 360-830 nm (471 samples each), the colour
system the reference renderer is built with (libSLR/defines.h:215-226).

The CIE table is standard data; the film-to-RGB conversion only matches the
reference's output files when its 16-bin discretisation starts from exactly
the same float32 values, so they are taken bit-for-bit from the reference's
single-precision table (libSLR/BasicTypes/spectrum_base.cpp, arrays
xbar/ybar/zbar_CIE1931_2deg).  The literals there are double constants
narrowed to float; ``np.float32(float(text))`` performs the same roundings.
The output stores each float as its bit pattern.

Usage: gen_cmf_table.py <reference spectrum_base.cpp> <output .inc>
"""
import re
import sys

import numpy as np


def table(text: str, name: str) -> list:
    m = re.search(name + r"\[\]\s*=\s*\{([^}]*)\}", text)
    vals = [np.float32(float(t)) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]
    assert len(vals) == 471, (name, len(vals))
    return vals


def main(src_path: str, out_path: str) -> None:
    text = open(src_path, encoding="utf-8-sig").read()
    out = ["// Generated by gen_cmf_table.py; CIE 1931 2-degree colour matching functions, 360-830 nm, 1 nm."]
    for axis in "xyz":
        vals = table(text, f"{axis}bar_CIE1931_2deg")
        out.append(f"static const unsigned int kCmf{axis.upper()}Bits[471] = {{")
        for i in range(0, 471, 8):
            out.append("    " + ", ".join("0x%08xu" % v.view(np.uint32) for v in vals[i:i + 8]) + ",")
        out.append("};")
    open(out_path, "w").write("\n".join(out) + "\n")


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
