#!/usr/bin/env python3
"""Build the reference renderer (SLR's ``libSLR``) as the CPU oracle.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``slr_gb300``) imports,
links or executes anything under ``oracle/``.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it,
and only as the checker / the timed CPU baseline.

Recipe
------
1. When the reference checkout is given (``--reference PATH`` or
   ``$SLR_REFERENCE``), the ``libSLR`` sources are copied into
   ``oracle/_ref/src`` and the build-only patches below are applied to that
   copy.  The reference tree itself is never written.  ``oracle/_ref`` is
   git-ignored.
2. Every translation unit is compiled with g++/gcc (no cmake, no external
   libraries) and linked, together with the oracle driver
   ``oracle/ref_driver.cpp`` and the no-op progress reporter
   ``oracle/progress_reporter_noop.cpp``, in two flavours:

   * ``check`` -> ``oracle/_ref/libslr_ref.so``: ``-O2 -ffp-contract=off``
     (P5), the checker of every parity test and golden fixture;
   * ``timing`` -> ``oracle/_ref/libslr_ref_timing.so``: the reference's own
     release flags ``-O3 -DNDEBUG`` (CMakeLists.txt:46-47) with the
     compiler's default contraction, timed as the CPU baseline.

On a machine without the reference checkout (the GPU host) step 1 is skipped
and the patched copy that travelled with the working tree is compiled.

Build-only patches (all applied to the copy):

* P1 ``libSLR/defines.h:106``: the Linux branch of ``SLR_memalign`` expands to
  an undeclared identifier; Linux is routed to the ``posix_memalign`` branch.
* P2 ``-include cstring``: ``Core/distributions.cpp:103,123,199`` use
  ``std::memcpy`` without including ``<cstring>``.
* P3 ``BasicTypes/spectrum_types.cpp:922-936``: the explicit specialisations
  of the static CMF members are declarations only; ``{}`` makes them
  definitions so the library links.
* P4 ``Core/surface_object.cpp:18`` and ``Core/medium_object.cpp:18`` include
  the SSE-only ``Accelerator/QBVH.h`` that nothing on the active path uses;
  the include is dropped so the library builds on aarch64 too.
* P5 ``-ffp-contract=off`` (check flavour only): x86-64 and aarch64 then round
  every operation the same way (no fused multiply-add), so golden dumps agree
  across hosts.
* P6 max depth: ``Renderer/PTRenderer.cpp:172`` caps a path at 100 vertices
  and ``Renderer/VolumetricPTRenderer.cpp:185`` has no cap.  Both now stop
  after ``slr_oracle_max_depth`` scattering vertices (a global the oracle driver,
  ``oracle/ref_driver.cpp``, sets), which is the ``maxDepth`` the GPU renderer implements.
* P7 ``Core/ProgressReporter.cpp`` is replaced by a no-op implementation (the
  stock one blocks up to 250 ms per progressive pass and can hang on a racy
  counter, ``Core/ProgressReporter.cpp:74-81,101-104``), and the progressive
  ``saveImage`` calls inside the render loops (``PTRenderer.cpp:84``,
  ``VolumetricPTRenderer.cpp:84``) are disabled so rendering writes no BMPs.
* P8 the message printed for each dropped non-finite sample
  (``PTRenderer.cpp:138``, ``VolumetricPTRenderer.cpp:138``) is replaced by an
  increment of a counter the oracle driver reports; which samples are dropped does
  not change.
* P9 ``Renderer/BPTRenderer.cpp``: a subpath stops after
  ``slr_oracle_max_depth`` vertices beyond its first (the stock renderer ends
  subpaths by Russian roulette only; the check sits before the BSDF sample
  at ``:347``, so the last vertex is still made and connected), the
  progressive ``saveImage`` (``:84``) is disabled and the message for a
  dropped non-finite connection (``:265``) becomes a counter increment.
* P10 ``Renderer/BPTRenderer.cpp:338``: a non-finite implicit-path
  contribution is dropped and counted instead of being added to the film
  (where one NaN would spoil the pixel for good).
* P11 ``Renderer/VolumetricBPTRenderer.cpp``: P9 and P10 for the volumetric
  bidirectional renderer (cap before the sample at ``:358``, ``:84``,
  ``:269``, ``:349``).
* P12 path tapes (test only): ``Core/random_number_generator.cpp:12-15``
  appends every 32-bit uniform it returns to ``slr_oracle_tape`` when the
  oracle driver has set it, and ``PTRenderer::Job::kernel`` (``PTRenderer.cpp:107``)
  calls ``slr_oracle_path_begin()`` before each pixel sample, so that a
  one-thread render records each path's uniforms in the reference's draw
  order; nothing changes while no tape is set.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
SRC_COPY = REF_OUT / "src" / "libSLR"
OBJ_DIR = REF_OUT / "obj"
LIB = REF_OUT / "libslr_ref.so"
FLAVORS = {
    "check": (["-O2", "-ffp-contract=off"], REF_OUT / "obj", LIB),
    "timing": (["-O3", "-DNDEBUG"], REF_OUT / "obj_timing", REF_OUT / "libslr_ref_timing.so"),
}
PATCH_SET = "P1 P2 P3 P4 P5 P6 P7 P8 P9 P10 P11 P12\n"

# Files excluded from the reference's own build (libSLR/CMakeLists.txt:45-51).
EXCLUDED = {
    "MemoryAllocators/StackAllocator.cpp", "MemoryAllocators/StackAllocator.h",
    "MemoryAllocators/MSpaceAllocator.cpp", "MemoryAllocators/MSpaceAllocator.h",
    "MemoryAllocators/dlmalloc.c", "MemoryAllocators/dlmalloc.h",
    "Renderer/AMCMCPPMRenderer.cpp", "Renderer/AMCMCPPMRenderer.h",
}
SOURCE_DIRS = ["", "External", "External/AnalyticSkyDomeRadiance", "MemoryAllocators",
               "BasicTypes", "Core", "RNG", "SurfaceShape", "MediumDistribution", "BSDF",
               "EDF", "PhaseFunction", "Texture", "SurfaceMaterial", "MediumMaterial",
               "Accelerator", "Camera", "Scene", "Renderer", "Helper"]


def _reference_root(reference: str | None = None) -> Path | None:
    path = reference or os.environ.get("SLR_REFERENCE")
    if not path:
        return None
    root = Path(path)
    return root if (root / "libSLR" / "defines.h").is_file() else None


def _replace_once(text: str, old: str, new: str, what: str) -> str:
    if text.count(old) < 1:
        raise RuntimeError(f"patch site not found: {what}")
    return text.replace(old, new)


def copy_and_patch(ref_root: Path) -> None:
    src = ref_root / "libSLR"
    if SRC_COPY.exists():
        shutil.rmtree(SRC_COPY)
    for d in SOURCE_DIRS:
        sdir = src / d
        if not sdir.is_dir():
            continue
        for f in sorted(sdir.iterdir()):
            if not f.is_file() or f.suffix not in (".h", ".hpp", ".cpp", ".c"):
                continue
            rel = f.relative_to(src).as_posix()
            if rel in EXCLUDED:
                continue
            dst = SRC_COPY / rel
            dst.parent.mkdir(parents=True, exist_ok=True)
            shutil.copyfile(f, dst)

    def patch(rel: str, fn) -> None:
        p = SRC_COPY / rel
        t = p.read_text(encoding="utf-8-sig")
        p.write_text(fn(t), encoding="utf-8")

    # P1
    patch("defines.h", lambda t: _replace_once(
        t, "#elif defined(SLR_Platform_OS_X) || defined(SLR_Platform_OpenBSD)\ninline void* SLR_memalign",
        "#elif defined(SLR_Platform_OS_X) || defined(SLR_Platform_OpenBSD) || defined(SLR_Platform_Linux)\ninline void* SLR_memalign",
        "P1 memalign"))
    # P3
    def p3(t: str) -> str:
        for real in ("float", "double"):
            for m in ("xbar", "ybar", "zbar"):
                t = _replace_once(t, f"DiscretizedSpectrumTemplate<{real}, NumStrataForStorage>::{m};",
                                  f"DiscretizedSpectrumTemplate<{real}, NumStrataForStorage>::{m}{{}};", "P3 " + m)
            t = _replace_once(t, f"DiscretizedSpectrumTemplate<{real}, NumStrataForStorage>::integralCMF;",
                              f"DiscretizedSpectrumTemplate<{real}, NumStrataForStorage>::integralCMF{{}};", "P3 integralCMF")
        return t
    patch("BasicTypes/spectrum_types.cpp", p3)
    # P4
    for rel in ("Core/surface_object.cpp", "Core/medium_object.cpp"):
        patch(rel, lambda t: _replace_once(t, '#include "../Accelerator/QBVH.h"', "", "P4 QBVH include"))
    # P6 + P7 (saveImage) + P8 (count dropped samples instead of printing them)
    decl = ("extern \"C\" unsigned int slr_oracle_max_depth;\n"
            "#include <atomic>\nextern std::atomic<unsigned long long> slr_oracle_dropped_samples;\n")
    drop_print = 'slrDevPrintf("Unexpected value detected: %s at (%f, %f)\\n", C.toString().c_str(), p.x, p.y);'
    drop_count = "slr_oracle_dropped_samples.fetch_add(1);"
    def p6_pt(t: str) -> str:
        t = _replace_once(t, "if (pathLength >= 100)", "if (pathLength > slr_oracle_max_depth)", "P6 PT")
        t = _replace_once(t, "            for (int lx = 0; lx < numPixelX; ++lx) {\n",
                          "            for (int lx = 0; lx < numPixelX; ++lx) {\n                slr_oracle_path_begin();\n",
                          "P12 PT path begin")
        t = _replace_once(t, "sensor->saveImage(filename,", "if (0) sensor->saveImage(filename,", "P7 PT")
        t = _replace_once(t, drop_print, drop_count, "P8 PT")
        return t.replace("namespace SLR {", decl + "namespace SLR {", 1)
    patch("Renderer/PTRenderer.cpp", lambda t: p6_pt(t).replace(
        "namespace SLR {", "extern \"C\" void slr_oracle_path_begin();\nnamespace SLR {", 1))
    def p12_rng(t: str) -> str:
        t = _replace_once(t, "        Types32bit::UInt fractionBits = (getUInt() >> 9) | 0x3f800000;\n"
                             "        return *(Types32bit::Float*)&fractionBits - 1.0f;",
                          "        Types32bit::UInt fractionBits = (getUInt() >> 9) | 0x3f800000;\n"
                          "        Types32bit::Float v = *(Types32bit::Float*)&fractionBits - 1.0f;\n"
                          "        if (slr_oracle_tape) slr_oracle_tape->push_back(v);\n"
                          "        return v;", "P12 rng tape")
        return t.replace("namespace SLR {", "#include <vector>\nextern std::vector<float>* slr_oracle_tape;\n"
                                            "namespace SLR {", 1)
    patch("Core/random_number_generator.cpp", p12_rng)
    def p6_vpt(t: str) -> str:
        t = _replace_once(t, "            ++pathLength;\n",
                          "            ++pathLength;\n            if (pathLength > slr_oracle_max_depth)\n                break;\n",
                          "P6 VolPT")
        t = _replace_once(t, "sensor->saveImage(filename,", "if (0) sensor->saveImage(filename,", "P7 VolPT")
        t = _replace_once(t, drop_print, drop_count, "P8 VolPT")
        return t.replace("namespace SLR {", decl + "namespace SLR {", 1)
    patch("Renderer/VolumetricPTRenderer.cpp", p6_vpt)
    def p9_bpt(t: str) -> str:
        t = _replace_once(t, "            BSDFQueryResult fsResult;\n            SampledSpectrum fs = bsdf->sample(",
                          "            if (vertices.size() > slr_oracle_max_depth)\n                break;\n"
                          "            BSDFQueryResult fsResult;\n            SampledSpectrum fs = bsdf->sample(", "P9 BPT cap")
        t = _replace_once(t, "sensor->saveImage(filename,", "if (0) sensor->saveImage(filename,", "P9 BPT save")
        t = _replace_once(t, 'slrDevPrintf("Unexpected value detected: %s at (%f, %f)\\n", contribution.toString().c_str(), p.x, p.y);',
                          "slr_oracle_dropped_samples.fetch_add(1);", "P9 BPT drop")
        t = _replace_once(t, "                    sensor->add(curPx, curPy, wls, contribution);",
                          "                    if (contribution.allFinite()) sensor->add(curPx, curPy, wls, contribution);\n"
                          "                    else slr_oracle_dropped_samples.fetch_add(1);", "P10 BPT implicit")
        return t.replace("namespace SLR {", decl + "namespace SLR {", 1)
    patch("Renderer/BPTRenderer.cpp", p9_bpt)
    def p11_vbpt(t: str) -> str:
        t = _replace_once(t, "            ABDFQueryResult* abdfResult;\n            SampledSpectrum abdfValue = abdf->sample(",
                          "            if (vertices.size() > slr_oracle_max_depth)\n                break;\n"
                          "            ABDFQueryResult* abdfResult;\n            SampledSpectrum abdfValue = abdf->sample(",
                          "P11 VBPT cap")
        t = _replace_once(t, "sensor->saveImage(filename,", "if (0) sensor->saveImage(filename,", "P11 VBPT save")
        t = _replace_once(t, 'slrDevPrintf("Unexpected value detected: %s at (%f, %f)\\n", contribution.toString().c_str(), p.x, p.y);',
                          "slr_oracle_dropped_samples.fetch_add(1);", "P11 VBPT drop")
        t = _replace_once(t, "                    sensor->add(curPx, curPy, wls, contribution);",
                          "                    if (contribution.allFinite()) sensor->add(curPx, curPy, wls, contribution);\n"
                          "                    else slr_oracle_dropped_samples.fetch_add(1);", "P11 VBPT implicit")
        return t.replace("namespace SLR {", decl + "namespace SLR {", 1)
    patch("Renderer/VolumetricBPTRenderer.cpp", p11_vbpt)
    # P7: the stock reporter is replaced by oracle/progress_reporter_noop.cpp
    (SRC_COPY / "Core" / "ProgressReporter.cpp").unlink()
    (REF_OUT / "src" / "PATCHED").write_text(PATCH_SET)


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stderr


def build(jobs: int | None = None, force: bool = False, verbose: bool = False, reference: str | None = None,
          flavors: tuple[str, ...] = ("check", "timing")) -> Path:
    """Builds the oracle library of every flavour (all translation units in
    one parallel pass); returns the check flavour's library."""
    ref_root = _reference_root(reference)
    marker = REF_OUT / "src" / "PATCHED"
    if ref_root is not None and (force or not marker.is_file() or marker.read_text() != PATCH_SET):
        copy_and_patch(ref_root)
        force = True
    if not (REF_OUT / "src" / "PATCHED").is_file():
        raise RuntimeError("reference sources unavailable: give the reference checkout (--reference or "
                           "$SLR_REFERENCE), or keep the patched copy in oracle/_ref/src")
    sources: list[tuple[Path, str]] = []
    for f in sorted(SRC_COPY.rglob("*")):
        if f.suffix in (".cpp", ".c"):
            sources.append((f, "lib"))
    sources.append((HERE / "progress_reporter_noop.cpp", "lib"))
    sources.append((HERE / "ref_driver.cpp", "driver"))
    cmds, links = [], []
    for flavor in flavors:
        opt, obj_dir, lib = FLAVORS[flavor]
        obj_dir.mkdir(parents=True, exist_ok=True)
        common = opt + ["-fPIC", "-w", "-pthread", f"-I{SRC_COPY}"]
        objs = []
        for f, kind in sources:
            if kind == "driver":
                tool = ["g++", "-std=gnu++14", "-include", "cstring", "-include", "cmath"] + common
            elif f.suffix == ".c":
                tool = ["gcc"] + common
            else:
                tool = ["g++", "-std=gnu++11", "-include", "cstring", "-include", "cmath"] + common
            rel = f.relative_to(SRC_COPY) if SRC_COPY in f.parents else Path("oracle") / f.name
            o = obj_dir / (rel.as_posix().replace("/", "__") + ".o")
            objs.append(o)
            if o.is_file() and o.stat().st_mtime >= f.stat().st_mtime and not force:
                continue
            cmds.append(tool + ["-c", str(f), "-o", str(o)])
        links.append((lib, objs))
    jobs = jobs or os.cpu_count() or 4
    failed = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for cmd, rc, err in ex.map(_compile, cmds):
            if rc != 0:
                failed.append((cmd, err))
            elif verbose:
                print(" ".join(cmd[-3:]))
    if failed:
        cmd, err = failed[0]
        raise RuntimeError(f"oracle compile failed ({len(failed)} units): {' '.join(cmd)}\n{err[-4000:]}")
    for lib, objs in links:
        if cmds or not lib.is_file():
            link = ["g++", "-shared", "-pthread", "-o", str(lib)] + [str(o) for o in objs]
            r = subprocess.run(link, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"oracle link failed:\n{r.stderr[-4000:]}")
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=None, help="reference checkout (default: $SLR_REFERENCE)")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    lib = build(jobs=a.j, force=a.force, verbose=a.v, reference=a.reference)
    print(f"built {lib} ({platform.machine()})")
    return 0


if __name__ == "__main__":
    sys.exit(main())
