"""Image-parity cases shared by the GPU image tests and the golden generator.

Each case names a procedural scene, the render settings, the integrator and
the number of independent batches on each side.  The reference side is the
reference renderer (the CPU oracle) run with ONE thread per batch: the
reference seeds one sampler per worker thread and hands tiles to threads as
they free up (PTRenderer.cpp:28-34, 60-78), so with several threads its film
depends on scheduling; with one thread a seed gives the same film on every
run.  Batches are independent seeds, so they may run in separate processes.

Small cases keep the reference statistics as committed fixtures
(tests/golden/images/<name>.npz, written by tests/golden/make_golden.py);
cases whose statistics would make large fixtures render the reference
batches when the test runs, in a process pool, with the same one-thread rule.

The GPU side is deterministic too (counter-based random numbers keyed by
seed, sample and pixel; films accumulated in sample order), so every verdict
is a fixed function of the fixed seeds below.
"""
from __future__ import annotations

import math
import multiprocessing as mp
import os
from dataclasses import dataclass

import numpy as np

GOLDEN_IMAGES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "images")


@dataclass(frozen=True)
class ImageCase:
    name: str
    scene: str                       # a constructor in slr_gb300.scenes
    scene_kw: tuple                  # its keyword arguments, as (key, value) pairs
    w: int
    h: int
    spp: int
    depth: int
    mode: str = "pt"                 # pt | vol | bpt | vbpt
    ref_batches: int = 64
    gpu_batches: int = 256
    ref_seed0: int = 1000
    gpu_seed0: int = 50000
    camera: str = ""                 # "" | thin_lens | equirect | bpt_equirect
    golden: bool = True              # reference statistics kept as a fixture
    frac_limit: float = 0.015

    def desc(self):
        from slr_gb300 import scenes
        d = getattr(scenes, self.scene)(**dict(self.scene_kw))
        if self.camera:
            d.camera = camera_override(self.camera, self.w, self.h)
        return d


def camera_override(kind: str, w: int, h: int):
    from slr_gb300.scene_desc import Camera
    from slr_gb300.scenes import look_at
    if kind == "thin_lens":
        return Camera("perspective", look_at((0.5, 0.5, 2.3), (0.5, 0.5, 0.0)), sensitivity=1.0, aspect=w / h,
                      fov_y=math.radians(38.0), lens_radius=0.04, img_plane_dist=1.0, obj_plane_dist=2.3)
    if kind == "equirect":
        return Camera("equirect", look_at((0.5, 0.45, 0.6), (0.5, 0.45, 0.0)), sensitivity=1.0,
                      phi_angle=2 * math.pi, theta_angle=math.pi)
    if kind == "bpt_equirect":
        return Camera("equirect", look_at((0.5, 0.5, 0.8), (0.5, 0.5, 0.0)), sensitivity=1.0,
                      phi_angle=math.radians(120.0), theta_angle=math.radians(90.0))
    raise ValueError(kind)


def _kw(**kw):
    return tuple(sorted(kw.items()))


HF_SMALL = dict(grid=24, spheres=5, sphere_freq=3, env_size=(64, 32))

CASES = {c.name: c for c in [
    # the closed box of the 256^2 benchmark configuration, at 32^2
    ImageCase("box_32", "box_scene", _kw(width=32, height=32), 32, 32, 8, 8, ref_batches=96, gpu_batches=192),
    # image sides that are not multiples of the 8 x 8 sensor tiles: the last
    # column and row also collect the overhanging tile positions
    ImageCase("ragged_box", "box_scene", _kw(width=21, height=13), 21, 13, 8, 8, ref_batches=256,
              gpu_batches=2048, ref_seed0=2000),
    ImageCase("ragged_ggx_ibl", "heightfield_scene", _kw(width=21, height=13, **HF_SMALL), 21, 13, 8, 3,
              ref_batches=1024, gpu_batches=8192, ref_seed0=3000, frac_limit=0.02),
    ImageCase("ggx_ibl_24", "heightfield_scene", _kw(width=24, height=24, **HF_SMALL), 24, 24, 8, 10,
              ref_batches=512, gpu_batches=1024, ref_seed0=4000, frac_limit=0.02),
    ImageCase("volumetric_20", "medium_box_scene", _kw(width=20, height=20, grid=32), 20, 20, 8, 32, mode="vol",
              ref_batches=128, gpu_batches=256, ref_seed0=5000, frac_limit=0.02),
    ImageCase("thin_lens", "box_scene", _kw(width=24, height=16), 24, 16, 8, 4, camera="thin_lens",
              ref_batches=128, gpu_batches=256, ref_seed0=6000),
    ImageCase("equirect", "box_scene", _kw(width=32, height=16), 32, 16, 8, 4, camera="equirect",
              ref_batches=128, gpu_batches=256, ref_seed0=7000),
    # bidirectional tracers against BPTRenderer / VolumetricBPTRenderer
    ImageCase("bpt_box", "box_scene", _kw(width=20, height=12), 20, 12, 8, 16, mode="bpt", ref_batches=96,
              gpu_batches=192, ref_seed0=8000, gpu_seed0=70000),
    ImageCase("bpt_every_bsdf", "glossy_box_scene", _kw(width=24, height=24), 24, 24, 8, 12, mode="bpt",
              ref_batches=96, gpu_batches=192, ref_seed0=9000, gpu_seed0=70000, frac_limit=0.02),
    ImageCase("bpt_thin_lens", "box_scene", _kw(width=16, height=16), 16, 16, 8, 12, mode="bpt",
              camera="thin_lens", ref_batches=96, gpu_batches=192, ref_seed0=10000, gpu_seed0=70000,
              frac_limit=0.02),
    ImageCase("bpt_equirect", "box_scene", _kw(width=16, height=16), 16, 16, 8, 12, mode="bpt",
              camera="bpt_equirect", ref_batches=96, gpu_batches=192, ref_seed0=11000, gpu_seed0=70000,
              frac_limit=0.02),
    ImageCase("bpt_env", "heightfield_scene", _kw(width=20, height=20, **HF_SMALL), 20, 20, 8, 8, mode="bpt",
              ref_batches=256, gpu_batches=512, ref_seed0=12000, gpu_seed0=70000, frac_limit=0.02),
    ImageCase("vbpt", "medium_box_scene", _kw(width=16, height=16, grid=16), 16, 16, 8, 16, mode="vbpt",
              ref_batches=96, gpu_batches=192, ref_seed0=13000, gpu_seed0=70000, frac_limit=0.02),
    # the benchmark configurations themselves: the 256^2 box at 16 spp and
    # depth 8, and the 256^3 fBm medium (16^3 super voxels) at a reduced
    # resolution; their statistics are rendered when the test runs
    ImageCase("c0_box_256", "box_scene", _kw(width=256, height=256), 256, 256, 16, 8, ref_batches=32,
              gpu_batches=128, ref_seed0=14000, golden=False),
    ImageCase("c3_medium_256", "medium_box_scene", _kw(width=48, height=48, grid=256), 48, 48, 8, 32, mode="vol",
              ref_batches=64, gpu_batches=256, ref_seed0=15000, golden=False, frac_limit=0.02),
]}


# ---------------------------------------------------------------------------
# reference side
# ---------------------------------------------------------------------------
_W = {}


def _worker_init(case: ImageCase, desc):
    from oracle import oracle as O
    if desc is None:          # large scenes: each worker builds its own copy
        desc = case.desc()
    _W["case"], _W["desc"] = case, desc
    _W["scene"] = None if case.mode in ("bpt", "vbpt") else O.RefScene(desc)


def _worker_batch(seed: int):
    from oracle import oracle as O
    c = _W["case"]
    if c.mode in ("bpt", "vbpt"):
        ref = O.RefScene(_W["desc"])          # one bidirectional render per reference sensor
        film, _ = ref.render_bpt(c.w, c.h, c.spp, c.depth, seed=seed, threads=1, volumetric=c.mode == "vbpt")
    else:
        ref = _W["scene"]
        film, _ = ref.render(c.w, c.h, c.spp, c.depth, seed=seed, threads=1, volumetric=c.mode == "vol")
    return seed, film.astype(np.float64) / c.spp, ref.last_dropped


def edge_sum(m: np.ndarray) -> float:
    """Sum of a batch estimate over the last column and the last row (the
    pixels that also collect the overhanging positions of the sensor's 8 x 8
    tiles when a side is not a multiple of 8)."""
    return float(m[:, -1].sum() + m[-1, :-1].sum())


def reference_stats(case: ImageCase, procs: int | None = None, desc=None) -> dict:
    """Mean and variance per pixel and film bin of the reference's batch
    estimates (film sum / spp), the per-batch image and edge sums and the
    dropped sample count, over seeds ref_seed0 .. ref_seed0 + ref_batches - 1,
    each rendered with one thread.  The result does not depend on `procs`.
    Without `desc`, every worker builds the case's scene itself."""
    procs = max(1, min(procs or os.cpu_count() or 1, case.ref_batches))
    seeds = list(range(case.ref_seed0, case.ref_seed0 + case.ref_batches))
    if procs == 1:
        _worker_init(case, desc)
        results = [_worker_batch(s) for s in seeds]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(procs, initializer=_worker_init, initargs=(case, desc)) as pool:
            results = pool.map(_worker_batch, seeds, chunksize=max(1, len(seeds) // (4 * procs)))
    results.sort(key=lambda r: r[0])
    m = np.stack([r[1] for r in results])
    return {"mean": m.mean(0), "var": m.var(0, ddof=1), "sums": m.reshape(len(m), -1).sum(1),
            "edge_sums": np.array([edge_sum(b) for b in m]), "batches": len(m),
            "dropped": int(sum(r[2] for r in results))}


def golden_path(case: ImageCase) -> str:
    return os.path.join(GOLDEN_IMAGES, case.name + ".npz")


def save_golden(case: ImageCase, st: dict) -> None:
    os.makedirs(GOLDEN_IMAGES, exist_ok=True)
    np.savez_compressed(golden_path(case), mean=st["mean"].astype(np.float32), var=st["var"].astype(np.float32),
                        sums=st["sums"], edge_sums=st["edge_sums"], batches=st["batches"], dropped=st["dropped"],
                        spp=case.spp, depth=case.depth, w=case.w, h=case.h, ref_seed0=case.ref_seed0)


def load_reference(case: ImageCase, desc=None) -> dict:
    """The reference statistics of a case: the committed fixture, or (cases
    without one) the reference rendered now."""
    if case.golden:
        g = np.load(golden_path(case))
        assert int(g["batches"]) == case.ref_batches and int(g["spp"]) == case.spp and int(g["depth"]) == case.depth
        return {"mean": g["mean"].astype(np.float64), "var": g["var"].astype(np.float64),
                "sums": g["sums"], "edge_sums": g["edge_sums"], "batches": int(g["batches"]),
                "dropped": int(g["dropped"])}
    return reference_stats(case, desc=desc)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def gpu_stats(gpu_lib, case: ImageCase, desc=None, batches: int | None = None) -> dict:
    desc = desc if desc is not None else case.desc()
    s = gpu_lib.Scene(desc)
    k = batches or case.gpu_batches
    acc = np.zeros((case.h, case.w, 16), np.float64)
    acc2 = np.zeros_like(acc)
    sums, edges, dropped = [], [], 0
    kw = {"bpt": case.mode in ("bpt", "vbpt"), "volumetric": case.mode in ("vol", "vbpt")}
    for i in range(k):
        film, st = s.render(case.w, case.h, case.spp, case.depth, seed=case.gpu_seed0 + i, **kw)
        dropped += st.dropped_samples
        m = film.astype(np.float64) / case.spp
        acc += m
        acc2 += m * m
        sums.append(m.sum())
        edges.append(edge_sum(m))
    s.close()
    mean = acc / k
    var = np.maximum(acc2 - k * mean * mean, 0.0) / (k - 1)
    return {"mean": mean, "var": var, "sums": np.array(sums), "edge_sums": np.array(edges), "batches": k,
            "dropped": dropped}


# ---------------------------------------------------------------------------
# the statistic
# ---------------------------------------------------------------------------
def _sum_z(a: np.ndarray, b: np.ndarray) -> float:
    return float((a.mean() - b.mean()) / math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b) + 1e-300))


def parity_report(g: dict, r: dict, ragged: bool = False) -> dict:
    """Per pixel and film bin: z = (mean_gpu - mean_ref) / se, se from the
    pooled batch variance of both sides (the hypothesis under test is that
    both run the same estimator, whose batch variance is then common; pooling
    also keeps a heavy-tailed bin's variance from resting on one side's
    batches alone).  frac = share of bins with |z| > 3 (0.27 % expected).
    gz = the difference of the per-batch image sums in standard errors (it
    takes the correlation between the 16 bins of one path into account).
    ragged: ez = the same for the sums over the last column and row, the
    pixels that also collect the overhanging tile positions (a bias of the
    edge clamp shows there)."""
    kg, kr = g["batches"], r["batches"]
    pooled = ((kg - 1) * g["var"] + (kr - 1) * r["var"]) / (kg + kr - 2)
    se = np.sqrt(pooled / kg + pooled / kr)
    diff = g["mean"] - r["mean"]
    zero = se == 0
    zero_ok = bool(np.all(np.abs(diff[zero]) < 1e-6))
    z = np.zeros_like(diff)
    z[~zero] = diff[~zero] / se[~zero]
    frac = float((np.abs(z[~zero]) > 3).mean()) if (~zero).any() else 0.0
    rep = {"frac": frac, "gz": _sum_z(g["sums"], r["sums"]), "bins": int((~zero).sum()),
           "zmax": float(np.abs(z).max()), "zero_bins_equal": zero_ok,
           "var_ratio": float(g["var"].sum() / max(r["var"].sum(), 1e-300))}
    if ragged:
        rep["ez"] = _sum_z(g["edge_sums"], r["edge_sums"])
    return rep


def assert_parity(rep: dict, frac_limit: float, name: str = "") -> None:
    msg = f"{name}: " + ", ".join(f"{k}={v:.4g}" if isinstance(v, float) else f"{k}={v}" for k, v in rep.items())
    assert rep["zero_bins_equal"], "bins that are zero on both sides' batches differ: " + msg
    assert rep["frac"] < frac_limit, "share of bins beyond 3 sigma too high: " + msg
    assert abs(rep["gz"]) < 4.0, "image sums differ: " + msg
    if "ez" in rep:
        assert abs(rep["ez"]) < 4.0, "bias along the clamped edge: " + msg
