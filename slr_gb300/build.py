"""Builds the CUDA extension ``slr_gb300/lib/libslrgpu.so`` for sm_103a.

Host C++ is compiled with g++ (-ffp-contract=off: the SBVH build, spectral
upsampling and environment tables must round exactly like the reference), the
kernels with nvcc for ``arch=compute_103a,code=sm_103a``; the translation
units compile in parallel and are linked by nvcc into one shared library
with a C ABI (include/slrgpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libslrgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["scene_host.cpp", "capi.cpp", "server.cpp"]
CUDA_SOURCES = ["render.cu", "bpt.cu"]


def _cuda_home() -> Path:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and (Path(c) / "bin" / "nvcc").exists():
            return Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stdout + r.stderr


def tuning_flags() -> list[str]:
    """nvcc flags of the tuned constants: SLRGPU_NVCC_EXTRA when set (the
    autotuner's candidates), else slr_gb300/tuning.json (the autotuner's
    choice), else none (the defaults in the sources)."""
    if "SLRGPU_NVCC_EXTRA" in os.environ:
        return os.environ["SLRGPU_NVCC_EXTRA"].split()
    tuning = PKG / "tuning.json"
    if not tuning.is_file():
        return []
    t = json.loads(tuning.read_text())
    flags = [f"-D{k}={int(v)}" for k, v in sorted(t.get("knobs", {}).items())]
    if "bvh_width" in t:
        flags.append(f"-DSLRGPU_BVH_WIDTH={int(t['bvh_width'])}")
    if "wave_paths" in t:
        flags.append(f"-DSLRGPU_WAVE_PATHS={int(t['wave_paths'])}u")
    return flags


# Library variants: the tuned build, and the same sources with 8-wide BVH
# nodes (the BVH width is a compile-time layout constant shared by the host
# collapse and the kernels; the 8-wide variant exists so that both widths are
# tested).  SLRGPU_LIB_VARIANT selects the one slr_gb300.api loads.
VARIANTS = {"": [], "w8": ["-DSLRGPU_BVH_WIDTH=8"]}


def lib_path(variant: str = "") -> Path:
    return LIB_DIR / (f"libslrgpu_{variant}.so" if variant else "libslrgpu.so")


def _variant_flags(variant: str, extra: list[str]) -> list[str]:
    flags = list(extra)
    if VARIANTS[variant]:
        flags = [f for f in flags if not f.startswith("-DSLRGPU_BVH_WIDTH=")] + VARIANTS[variant]
    return flags


def build(verbose: bool = False, force: bool = False, extra_nvcc: list[str] | None = None,
          variants: tuple[str, ...] = ("", "w8")) -> Path:
    """Compiles every translation unit of every variant in one parallel pass
    and links each variant's shared library; returns the default library."""
    base_flags = list(extra_nvcc or []) + tuning_flags()
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    LIB_DIR.mkdir(exist_ok=True)
    inc = [f"-I{cuda / 'include'}", f"-I{CSRC}"]
    deps = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.inc")) + \
        [PKG.parent / "include" / "slrgpu.h"]
    newest_dep = max(p.stat().st_mtime for p in deps)
    jobs, links = [], []
    for variant in variants:
        flags = _variant_flags(variant, base_flags)
        bdir = BUILD if not variant else PKG / f"_build_{variant}"
        bdir.mkdir(exist_ok=True)
        # rebuild the objects when the flags change
        stamp = bdir / "nvcc_flags"
        vforce = force or not stamp.is_file() or stamp.read_text() != " ".join(flags)
        # layout constants the host build shares with the kernels (BVH width)
        host_defs = [f for f in flags if f.startswith("-DSLRGPU_BVH_WIDTH=")]
        objs, vjobs = [], []
        for src in HOST_SOURCES:
            o = bdir / (src + ".o")
            objs.append(o)
            sp = CSRC / src
            if vforce or not o.exists() or o.stat().st_mtime < max(sp.stat().st_mtime, newest_dep):
                vjobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                              *host_defs, *inc, "-c", str(sp), "-o", str(o)])
        for src in CUDA_SOURCES:
            o = bdir / (src + ".o")
            objs.append(o)
            sp = CSRC / src
            if vforce or not o.exists() or o.stat().st_mtime < max(sp.stat().st_mtime, newest_dep):
                vjobs.append([nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
                              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v", *flags,
                              *inc, "-c", str(sp), "-o", str(o)])
        jobs += vjobs
        links.append((variant, objs, stamp, flags, bool(vjobs)))
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, rc, out in ex.map(_run, jobs):
            if rc != 0:
                raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{out[-6000:]}")
            if verbose:
                print(out)
    for variant, objs, stamp, flags, rebuilt in links:
        stamp.write_text(" ".join(flags))
        lib = lib_path(variant)
        if rebuilt or not lib.exists():
            cmd = [nvcc, "-shared", *ARCH, "-o", str(lib), *[str(o) for o in objs], "-lcudart_static", "-lrt",
                   "-lpthread", "-ldl"]
            _, rc, out = _run(cmd)
            if rc != 0:
                raise RuntimeError(f"link failed: {' '.join(cmd)}\n{out[-6000:]}")
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
