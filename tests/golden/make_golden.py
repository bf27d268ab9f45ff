#!/usr/bin/env python3
"""Generates the golden fixtures in tests/golden/ from the CPU oracle (the
reference renderer built by oracle/build_ref.py).  Run from the repository
root:  python tests/golden/make_golden.py

* images/<case>.npz - for every image case of tests/image_cases.py that
  keeps a fixture: per pixel and film bin the mean and variance of the
  reference renderer's independent batch estimates (film sum / spp of each
  batch, one seed and ONE render thread per batch, so the numbers do not
  depend on scheduling), the per-batch image sums and edge sums, and the
  dropped-sample count.
* trace_box.npz, trace_soup.npz - ray sets with the reference SBVH's closest
  hit (prim, t) and any-hit result.
* bsdf_kat.npz - reference BSDF sample / evaluate / pdf results at fixed
  (query, sample) tuples.
"""
import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from slr_gb300 import scenes  # noqa: E402
from tests import helpers  # noqa: E402
from tests.bsdf_cases import bsdf_cases  # noqa: E402
from tests import image_cases  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")


def make_images(names):
    for name in names:
        case = image_cases.CASES[name]
        st = image_cases.reference_stats(case)
        image_cases.save_golden(case, st)
        print(f"{name}: {st['batches']} batches, image sum {st['sums'].mean():.6g}, dropped {st['dropped']}")


def make_rays():
    for name, d, n in (("trace_box", scenes.box_scene(32, 32), 20000), ("trace_soup", helpers.triangle_soup(3000, 7), 20000)):
        rays = helpers.random_rays(d, n, seed=11)
        ref = O.RefScene(d)
        prim, t, b1, b2 = ref.trace(rays)
        occ, _, _, _ = ref.trace(rays, anyhit=True)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), rays=rays, prim=prim, t=t, b1=b1, b2=b2, occluded=occ)


def make_bsdfs():
    kat = {}
    for case in bsdf_cases():
        out = O.bsdf_query(case["kind"], case["spec0"], case.get("spec1"), case.get("spec2"), case.get("ax", 0.0),
                           case.get("ay", 0.0), case["queries"])
        kat[case["name"]] = out
    np.savez_compressed(os.path.join(OUT, "bsdf_kat.npz"), **kat)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("images", nargs="*", help="image cases to regenerate (default: every case with a fixture)")
    ap.add_argument("--rays-and-bsdfs", action="store_true", help="also regenerate the ray and BSDF fixtures")
    ap.add_argument("--bsdfs-only", action="store_true", help="regenerate the BSDF fixture alone")
    a = ap.parse_args()
    if a.bsdfs_only:
        make_bsdfs()
    else:
        names = a.images or [n for n, c in image_cases.CASES.items() if c.golden]
        make_images(names)
        if a.rays_and_bsdfs:
            make_rays()
            make_bsdfs()
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
