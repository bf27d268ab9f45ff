#!/usr/bin/env python3
"""Generates the golden fixtures in tests/golden/ from the CPU oracle (the
reference renderer built by oracle/build_ref.py).  Run from the repository
root:  python tests/golden/make_golden.py

* box_render_32.npz - reference PTRenderer on the box scene at 32x32, max
  depth 8: per pixel and film bin the mean and variance of K independent
  batch estimates (film sum / spp of each batch), for the statistical image
  parity test.
* trace_box.npz, trace_soup.npz - ray sets with the reference SBVH's closest
  hit (prim, t) and any-hit result.
* bsdf_kat.npz - reference BSDF sample / evaluate / pdf results at fixed
  (query, sample) tuples.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from slr_gb300 import scenes  # noqa: E402
from tests import helpers  # noqa: E402
from tests.bsdf_cases import bsdf_cases  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")


def render_batches(desc, w, h, spp, depth, batches, seed0=1000):
    ref = O.RefScene(desc)
    means = []
    for k in range(batches):
        film, _ = ref.render(w, h, spp, depth, seed=seed0 + k, threads=os.cpu_count())
        means.append(film / spp)
    m = np.stack(means).astype(np.float64)
    return m.mean(0), m.var(0, ddof=1)


def main():
    desc = scenes.box_scene(32, 32)
    K, spp = 48, 8
    mean, var = render_batches(desc, 32, 32, spp, 8, K)
    np.savez_compressed(os.path.join(OUT, "box_render_32.npz"), mean=mean.astype(np.float32),
                        var=var.astype(np.float32), batches=K, spp=spp, max_depth=8)
    for name, d, n in (("trace_box", scenes.box_scene(32, 32), 20000), ("trace_soup", helpers.triangle_soup(3000, 7), 20000)):
        rays = helpers.random_rays(d, n, seed=11)
        ref = O.RefScene(d)
        prim, t, b1, b2 = ref.trace(rays)
        occ, _, _, _ = ref.trace(rays, anyhit=True)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), rays=rays, prim=prim, t=t, b1=b1, b2=b2, occluded=occ)
    kat = {}
    for case in bsdf_cases():
        out = O.bsdf_query(case["kind"], case["spec0"], case.get("spec1"), case.get("spec2"), case.get("ax", 0.0),
                           case.get("ay", 0.0), case["queries"])
        kat[case["name"]] = out
    np.savez_compressed(os.path.join(OUT, "bsdf_kat.npz"), **kat)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
