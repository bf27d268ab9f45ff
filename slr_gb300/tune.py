"""Autotuner for the compile-time occupancy targets and the wave size.

Each candidate rebuilds the CUDA library with its nvcc flags and times a
short render of a workload in a fresh process; the fastest flags are written
to ``slr_gb300/tuning.json``, which ``slr_gb300/build.py`` applies by default
(the environment variable SLRGPU_NVCC_EXTRA overrides it).  The search is a
coordinate descent over the knobs: one knob at a time, the others held at
their best value so far.

    python -m slr_gb300.tune [--workload small|ggx_ibl_1m|volumetric_small] [--rounds 1]

Each workload tunes the knobs of the kernels it runs; tuning.json keeps the
other knobs as they were.

Knobs (resident blocks of 256 threads per SM the kernels are compiled for):
SLRGPU_TRACE_MIN_BLOCKS (closest/any-hit traversal), SLRGPU_SHADE_MIN_BLOCKS
(surface shading), SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS (GGX dielectric
shading), SLRGPU_SHADEVOL_MIN_BLOCKS (volumetric shading),
SLRGPU_MEDIUM_MIN_BLOCKS (medium transmittance); the paths per wave; and
the BVH width (4 or 8 children per node, host build and kernels alike).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
TUNING = PKG / "tuning.json"

KNOBS = {
    "SLRGPU_TRACE_MIN_BLOCKS": [3, 4, 5],
    "SLRGPU_SHADE_MIN_BLOCKS": [2, 3, 4],
    "SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS": [2, 3, 4],
    "SLRGPU_SHADEVOL_MIN_BLOCKS": [2, 3],
    "SLRGPU_MEDIUM_MIN_BLOCKS": [2, 3, 4],
    "SLRGPU_VOLINTERACT_MIN_BLOCKS": [2, 3, 4],
}
DEFAULTS = {"SLRGPU_TRACE_MIN_BLOCKS": 4, "SLRGPU_SHADE_MIN_BLOCKS": 3, "SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS": 3,
            "SLRGPU_SHADEVOL_MIN_BLOCKS": 3, "SLRGPU_MEDIUM_MIN_BLOCKS": 4, "SLRGPU_VOLINTERACT_MIN_BLOCKS": 3,
            "wave_paths": 1 << 22, "bvh_width": 4}   # the sources' defaults
WAVE_PATHS = [1 << 22, 1 << 23, 1 << 24, 1 << 25, 1 << 26]
BVH_WIDTHS = [4, 8]
# The knobs a workload exercises (a knob of kernels the workload never
# launches would only be tuned to noise).
WORKLOAD_KNOBS = {
    "small": ["bvh_width", "SLRGPU_TRACE_MIN_BLOCKS", "SLRGPU_SHADE_MIN_BLOCKS",
              "SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS", "wave_paths"],
    "ggx_ibl_1m": ["bvh_width", "SLRGPU_TRACE_MIN_BLOCKS", "SLRGPU_SHADE_MIN_BLOCKS",
                   "SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS", "wave_paths"],
    "volumetric_small": ["SLRGPU_VOLINTERACT_MIN_BLOCKS", "SLRGPU_SHADEVOL_MIN_BLOCKS", "SLRGPU_MEDIUM_MIN_BLOCKS"],
}

# The timed workload of each candidate: scene recipe, size, spp, depth, integrator.
WORKLOADS = {
    "small": "scenes.heightfield_scene(grid=256, spheres=16, sphere_freq=12, env_size=(256, 128), width=512, "
             "height=512), 512, 512, 8, 10, False",
    "ggx_ibl_1m": "scenes.heightfield_scene(seed=0), 1024, 1024, 64, 10, False",
    "volumetric_small": "scenes.medium_box_scene(256, 256, grid=128), 256, 256, 8, 32, True",
}

_TIMER = r"""
import sys, time
sys.path.insert(0, {root!r})
from slr_gb300 import api, scenes
desc, w, h, spp, depth, vol = {workload}
scene = api.Scene(desc)
spw = max(1, {paths} // (((w + 7) // 8 * 8) * ((h + 7) // 8 * 8)))
best = 0.0
for i in range(3):
    _, st = scene.render(w, h, spp, depth, seed=i, volumetric=vol, samples_per_wave=min(spw, spp))
    if i:
        best = max(best, st.path_samples / st.kernel_seconds)
print(best)
"""


def _flags(cfg: dict) -> list[str]:
    flags = [f"-D{k}={v}" for k, v in sorted(cfg.items()) if k in KNOBS]
    if "bvh_width" in cfg:
        flags.append(f"-DSLRGPU_BVH_WIDTH={int(cfg['bvh_width'])}")
    return flags


def measure(cfg: dict, workload: str) -> float:
    env = dict(os.environ, SLRGPU_NVCC_EXTRA=" ".join(_flags(cfg)))
    subprocess.run([sys.executable, str(PKG / "build.py"), "--force"], env=env, check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    code = _TIMER.format(root=str(ROOT), workload=WORKLOADS[workload], paths=cfg.get("wave_paths", 1 << 22))
    out = subprocess.run([sys.executable, "-c", code], env=env, check=True, capture_output=True, text=True)
    return float(out.stdout.strip().splitlines()[-1])


def load() -> dict:
    if TUNING.is_file():
        return json.loads(TUNING.read_text())
    return {}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="small", choices=sorted(WORKLOADS))
    ap.add_argument("--rounds", type=int, default=1)
    args = ap.parse_args()
    prev = load()
    best = dict(DEFAULTS)
    best.update({k: v for k, v in prev.get("knobs", {}).items() if k in KNOBS})
    best["wave_paths"] = prev.get("wave_paths", DEFAULTS["wave_paths"])
    best["bvh_width"] = prev.get("bvh_width", DEFAULTS["bvh_width"])
    log = []
    best_val = measure(best, args.workload)
    log.append({"config": dict(best), "samples_per_s": best_val})
    space = dict(KNOBS, wave_paths=WAVE_PATHS, bvh_width=BVH_WIDTHS)
    for _ in range(args.rounds):
        for knob in WORKLOAD_KNOBS[args.workload]:
            values = space[knob]
            for v in values:
                if v == best[knob]:
                    continue
                cand = dict(best, **{knob: v})
                val = measure(cand, args.workload)
                log.append({"config": cand, "samples_per_s": val})
                print(json.dumps(log[-1]), flush=True)
                if val > best_val * 1.01:
                    best, best_val = cand, val
    runs = dict(prev.get("runs", {}))
    runs[args.workload] = {"samples_per_s": best_val, "trials": log}
    result = {"knobs": {k: best[k] for k in KNOBS}, "wave_paths": best["wave_paths"], "bvh_width": best["bvh_width"],
              "runs": runs}
    TUNING.write_text(json.dumps(result, indent=1) + "\n")
    # rebuild with the chosen flags
    subprocess.run([sys.executable, str(PKG / "build.py"), "--force"], check=True, stdout=subprocess.DEVNULL)
    print(json.dumps({"knobs": result["knobs"], "wave_paths": result["wave_paths"], "bvh_width": result["bvh_width"],
                      "samples_per_s": best_val}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
