#!/usr/bin/env python3
"""Generates ``upsampling_table.inc``: the RGB -> spectrum upsampling table
of Meng et al. 2015, "Physically Meaningful Rendering using Tristimulus
Colours" (EGSR), as used by the reference renderer.

The table is data, not code: a 12 x 14 grid over Meng's (u, v) chromaticity
plane whose cells list up to six data points, and one 95-sample spectrum
(360-830 nm, X+Y+Z = 1) per data point.  Renders are only comparable with the
reference when RGB-defined reflectances, emitters and environment texels turn
into exactly the same spectra, so the float32 values are reproduced
bit-for-bit from the reference's single-precision table
(libSLR/BasicTypes/spectrum_types.cpp:1003-1175 for the grid,
:1178-1365 for the data points).  The literals there are double constants
narrowed to float by the compiler; ``np.float32(float(text))`` performs the
same two roundings.  The output stores each float as its bit pattern.

Usage: gen_upsampling_table.py <reference spectrum_types.cpp> <output .inc>
"""
import re
import sys

import numpy as np


def main(src_path: str, out_path: str) -> None:
    lines = open(src_path, encoding="utf-8-sig").read().split("\n")
    grid_start = next(i for i, l in enumerate(lines)
                      if "UpsampledContinuousSpectrumTemplate<float, NumSpectralSamples>::spectrum_grid[] = {" in l)
    pts_start = next(i for i, l in enumerate(lines)
                     if "UpsampledContinuousSpectrumTemplate<float, NumSpectralSamples>::spectrum_data_points[] = {" in l)
    cells = []
    for l in lines[grid_start + 1:]:
        if l.strip().startswith("};"):
            break
        m = re.match(r"\s*\{\s*(\d+),\s*(\d+),\s*\{([^}]*)\}\s*\}", l)
        if not m:
            continue
        idx = [255 if t.strip() == "UINT8_MAX" else int(t) for t in m.group(3).split(",")]
        cells.append([int(m.group(1)), int(m.group(2))] + idx)
    points_uv, points_spec = [], []
    for l in lines[pts_start + 1:]:
        if l.strip().startswith("};"):
            break
        groups = re.findall(r"\{([^{}]*)\}", l)
        if len(groups) != 3:
            continue
        uv = [np.float32(float(t)) for t in groups[1].split(",")]
        sp = [np.float32(float(t)) for t in groups[2].split(",")]
        assert len(uv) == 2 and len(sp) == 95, (len(uv), len(sp))
        points_uv.append(uv)
        points_spec.append(sp)
    assert len(cells) == 12 * 14, len(cells)

    def bits(v):
        return "0x%08xu" % np.float32(v).view(np.uint32)

    out = ["// Generated by gen_upsampling_table.py; Meng et al. 2015 spectral upsampling data.",
           f"// {len(cells)} grid cells, {len(points_uv)} data points of 95 samples (360-830 nm).",
           f"#define SLRGPU_UPS_NUM_POINTS {len(points_uv)}",
           "static const unsigned char kUpsGridCells[168][8] = {"]
    for c in cells:
        out.append("    {" + ", ".join(str(v) for v in c) + "},")
    out.append("};")
    out.append(f"static const unsigned int kUpsPointUVBits[{len(points_uv)}][2] = {{")
    for uv in points_uv:
        out.append("    {" + ", ".join(bits(v) for v in uv) + "},")
    out.append("};")
    out.append(f"static const unsigned int kUpsPointSpectrumBits[{len(points_uv)}][95] = {{")
    for sp in points_spec:
        out.append("    {" + ", ".join(bits(v) for v in sp) + "},")
    out.append("};")
    open(out_path, "w").write("\n".join(out) + "\n")


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
