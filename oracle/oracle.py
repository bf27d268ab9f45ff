"""ctypes binding of the CPU oracle (the reference's own libSLR, built by
``oracle/build_ref.py``).  TEST INFRASTRUCTURE ONLY: used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the
checker / the timed CPU baseline, never by the product path.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libslr_ref.so"
# the reference's release-flag build (-O3 -DNDEBUG), timed as the CPU
# baseline; every parity check uses LIB_PATH
TIMING_LIB_PATH = HERE / "_ref" / "libslr_ref_timing.so"

_lib = None
_libc = None


@contextlib.contextmanager
def _quiet():
    """Sends the reference's progress lines (``slrprintf`` of the renderers
    and of the SBVH build, which go to the C stdout) to /dev/null for the
    duration of a call, unless SLR_ORACLE_VERBOSE is set."""
    global _libc
    if os.environ.get("SLR_ORACLE_VERBOSE"):
        yield
        return
    if _libc is None:
        _libc = C.CDLL(None)
    sys.stdout.flush()
    _libc.fflush(None)
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(devnull, 1)
        yield
    finally:
        _libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


def available() -> bool:
    return LIB_PATH.is_file()


_flavor = "check"


def use_timing_build() -> None:
    """Loads the release-flag build instead of the checker build; only before
    the first call into the oracle of this process (the CPU-baseline legs)."""
    global _flavor
    if _lib is not None and _flavor != "timing":
        raise RuntimeError("the oracle's checker build is already loaded in this process")
    _flavor = "timing"


def lib():
    global _lib
    if _lib is None:
        path = TIMING_LIB_PATH if _flavor == "timing" else LIB_PATH
        if not path.is_file():
            raise RuntimeError(f"oracle library missing: {path} (run oracle/build_ref.py)")
        L = C.CDLL(str(path))
        P, I, F, D = C.c_void_p, C.c_int, C.c_float, C.c_double
        fp, up, dp = C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_double)
        hp = C.POINTER(C.c_uint16)
        sig = {
            "ora_scene_new": (P, []),
            "ora_scene_free": (None, [P]),
            "ora_spectrum_rgb": (I, [P, I, F, F, F]),
            "ora_spectrum_regular": (I, [P, F, F, fp, I]),
            "ora_spectrum_irregular": (I, [P, fp, fp, I]),
            "ora_material_matte": (I, [P, I]),
            "ora_material_specular_reflection": (I, [P, I, I, I]),
            "ora_material_specular_scattering": (I, [P, I, I, I]),
            "ora_material_microfacet_reflection": (I, [P, I, I, F, F]),
            "ora_material_microfacet_scattering": (I, [P, I, I, F, F]),
            "ora_material_emitter": (I, [P, I, I]),
            "ora_mesh": (I, [P, fp, fp, fp, fp, I, up, I, I]),
            "ora_env_ibl": (I, [P, hp, I, I, F]),
            "ora_camera_perspective": (I, [P, fp, F, F, F, F, F, F]),
            "ora_medium_density_grid": (I, [P, fp, fp, I, I, fp, I, I, I, F]),
            "ora_camera_equirect": (I, [P, fp, F, F, F]),
            "ora_build": (I, [P]),
            "ora_render": (I, [P, I, I, I, I, I, I, I, fp, dp]),
            "ora_render_bpt": (I, [P, I, I, I, I, I, I, I, fp, dp]),
            "ora_render_record": (I, [P, I, I, I, I, fp, fp, C.c_uint32, up, C.c_uint32, up, up]),
            "ora_sbvh_build": (I, [P, up, up, fp, up]),
            "ora_sbvh_dump": (I, [P, fp, up, up]),
            "ora_trace": (I, [P, fp, I, I, I, up, fp, fp, fp]),
            "ora_bsdf_query": (I, [I, fp, fp, fp, F, F, fp, I, fp]),
            "ora_spectrum_eval": (I, [P, I, fp, I, fp]),
            "ora_dropped_samples": (C.c_ulonglong, []),
            "ora_medium_query": (I, [P, I, I, fp, fp, C.POINTER(C.c_int), up, I, fp]),
            "ora_film_bmp": (I, [fp, I, I, F, F, C.c_char_p]),
            "ora_film_cmf": (I, [fp, fp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _f(a):
    a = np.ascontiguousarray(a, np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def _u(a):
    a = np.ascontiguousarray(a, np.uint32)
    return a, a.ctypes.data_as(C.POINTER(C.c_uint32))


class RefScene:
    """A scene built inside the reference library from a SceneDesc."""

    def __init__(self, desc, build: bool = True, library=None):
        """library: another implementation of the ora_* scene-building calls
        with the same signatures (the shim test application); the oracle by
        default."""
        L = library if library is not None else lib()
        self._L = L
        self.desc = desc
        self.h = L.ora_scene_new()
        keep = []
        sp_ids = []
        for sp in desc.spectra:
            if sp.kind == "rgb":
                sp_ids.append(L.ora_spectrum_rgb(self.h, sp.sp_type, *sp.rgb))
            elif sp.kind == "regular":
                v, vp = _f(sp.values)
                keep.append(v)
                sp_ids.append(L.ora_spectrum_regular(self.h, sp.min_wl, sp.max_wl, vp, len(v)))
            elif sp.kind == "irregular":
                w, wp = _f(sp.wavelengths)
                v, vp = _f(sp.values)
                keep += [w, v]
                sp_ids.append(L.ora_spectrum_irregular(self.h, wp, vp, len(v)))
            else:
                raise ValueError(sp.kind)
        self.spectrum_ids = sp_ids
        mat_ids = []
        for m in desc.materials:
            s = [sp_ids[i] for i in m.spectra]
            if m.kind == "matte":
                mid = L.ora_material_matte(self.h, s[0])
            elif m.kind == "specular_reflection":
                mid = L.ora_material_specular_reflection(self.h, *s)
            elif m.kind == "specular_scattering":
                mid = L.ora_material_specular_scattering(self.h, *s)
            elif m.kind == "microfacet_reflection":
                mid = L.ora_material_microfacet_reflection(self.h, s[0], s[1], m.alpha_x, m.alpha_y)
            elif m.kind == "microfacet_scattering":
                mid = L.ora_material_microfacet_scattering(self.h, s[0], s[1], m.alpha_x, m.alpha_y)
            elif m.kind == "emitter":
                mid = L.ora_material_emitter(self.h, mat_ids[m.base], s[0])
            else:
                raise ValueError(m.kind)
            mat_ids.append(mid)
        for mesh in desc.meshes:
            p, pp = _f(mesh.positions)
            n, np_ = _f(mesh.normals)
            t, tp = _f(mesh.tangents)
            uv, uvp = _f(mesh.uvs)
            idx, ip = _u(mesh.indices)
            rc = L.ora_mesh(self.h, pp, np_, tp, uvp, len(p), ip, len(idx), mat_ids[mesh.material])
            if rc < 0:
                raise ValueError("invalid mesh")
        if desc.environment is not None:
            img = np.ascontiguousarray(desc.environment.rgba_half, np.float16).view(np.uint16)
            keep.append(img)
            L.ora_env_ibl(self.h, img.ctypes.data_as(C.POINTER(C.c_uint16)), img.shape[1], img.shape[0],
                          desc.environment.scale)
        if desc.medium is not None:
            md = desc.medium
            bmin, bminp = _f(md.bounds_min)
            bmax, bmaxp = _f(md.bounds_max)
            dens, densp = _f(md.density)
            keep += [bmin, bmax, dens]
            nz, ny, nx = dens.shape
            L.ora_medium_density_grid(self.h, bminp, bmaxp, sp_ids[md.sigma_s], sp_ids[md.sigma_e], densp, nx, ny, nz,
                                      md.hg_g)
        cam = desc.camera
        if cam is not None:
            m, mp = _f(cam.cam_to_world)
            keep.append(m)
            if cam.kind == "perspective":
                L.ora_camera_perspective(self.h, mp, cam.sensitivity, cam.aspect, cam.fov_y, cam.lens_radius,
                                         cam.img_plane_dist, cam.obj_plane_dist)
            else:
                L.ora_camera_equirect(self.h, mp, cam.sensitivity, cam.phi_angle, cam.theta_angle)
        self._keep = keep
        if build:
            with _quiet():
                L.ora_build(self.h)

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_L", None) is not None:
            self._L.ora_scene_free(self.h)
            self.h = None

    def render(self, width, height, spp, max_depth, seed=0, threads=None, volumetric=False):
        """Returns (film sum (h, w, 16) float32, render seconds)."""
        threads = threads or os.cpu_count() or 1
        film = np.zeros((height, width, 16), np.float32)
        sec = C.c_double(0)
        with _quiet():
            rc = lib().ora_render(self.h, int(volumetric), spp, max_depth, width, height, threads, seed,
                                  film.ctypes.data_as(C.POINTER(C.c_float)), C.byref(sec))
        if rc != 0:
            raise RuntimeError("oracle render failed")
        self.last_dropped = int(lib().ora_dropped_samples())
        return film, sec.value

    def render_record(self, width, height, max_depth, seed=0):
        """One sample per pixel with one thread, recording every path's
        uniforms (build patch P12).  Returns (film (h, w, 16), tapes): tapes[k]
        is the float32 array of the k-th path's draws, paths in the
        renderer's order (8 x 8 tiles row by row, pixels row by row within a
        tile)."""
        film = np.zeros((height, width, 16), np.float32)
        cap_draws, cap_paths = 1 << 16, 1 << 10
        while True:
            tape = np.zeros(cap_draws, np.float32)
            starts = np.zeros(cap_paths, np.uint32)
            nd, npaths = C.c_uint32(), C.c_uint32()
            with _quiet():
                rc = lib().ora_render_record(self.h, max_depth, width, height, seed,
                                             film.ctypes.data_as(C.POINTER(C.c_float)),
                                             tape.ctypes.data_as(C.POINTER(C.c_float)), cap_draws,
                                             starts.ctypes.data_as(C.POINTER(C.c_uint32)), cap_paths,
                                             C.byref(nd), C.byref(npaths))
            if rc == -3:
                cap_draws, cap_paths = max(cap_draws, nd.value), max(cap_paths, npaths.value)
                continue
            if rc != 0:
                raise RuntimeError("oracle render failed")
            break
        bounds = list(starts[:npaths.value]) + [nd.value]
        tapes = [tape[bounds[k]:bounds[k + 1]].copy() for k in range(npaths.value)]
        return film, tapes

    def render_bpt(self, width, height, spp, max_depth, seed=0, threads=None, volumetric=False):
        """BPTRenderer (VolumetricBPTRenderer with volumetric=True): returns
        (film sum (h, w, 16) float32, render seconds).  One BPT render per
        RefScene (the reference's sensor cannot take a second one)."""
        threads = threads or os.cpu_count() or 1
        film = np.zeros((height, width, 16), np.float32)
        sec = C.c_double(0)
        with _quiet():
            rc = lib().ora_render_bpt(self.h, int(volumetric), spp, max_depth, width, height, threads, seed,
                                      film.ctypes.data_as(C.POINTER(C.c_float)), C.byref(sec))
        if rc == -2:
            raise RuntimeError("one BPT render per oracle scene")
        if rc != 0:
            raise RuntimeError("oracle BPT render failed")
        self.last_dropped = int(lib().ora_dropped_samples())
        return film, sec.value

    def sbvh_stats(self):
        nf, dep, nn = C.c_uint32(), C.c_uint32(), C.c_uint32()
        cost = C.c_float()
        with _quiet():
            lib().ora_sbvh_build(self.h, C.byref(nf), C.byref(dep), C.byref(cost), C.byref(nn))
        return {"fragments": nf.value, "depth": dep.value, "cost": cost.value, "nodes": nn.value}

    def sbvh_dump(self):
        st = self.sbvh_stats()
        boxes = np.zeros((st["nodes"], 6), np.float32)
        words = np.zeros((st["nodes"], 5), np.uint32)
        leaves = np.zeros(st["fragments"], np.uint32)
        lib().ora_sbvh_dump(self.h, boxes.ctypes.data_as(C.POINTER(C.c_float)),
                            words.ctypes.data_as(C.POINTER(C.c_uint32)),
                            leaves.ctypes.data_as(C.POINTER(C.c_uint32)))
        return boxes, words, leaves

    def trace(self, rays: np.ndarray, anyhit: bool = False, threads=None):
        """rays: (n, 8) float32 (org, tmin, dir, tmax)."""
        threads = threads or os.cpu_count() or 1
        r, rp = _f(rays)
        n = len(r)
        prim = np.zeros(n, np.uint32)
        t = np.zeros(n, np.float32)
        b1 = np.zeros(n, np.float32)
        b2 = np.zeros(n, np.float32)
        with _quiet():
            lib().ora_trace(self.h, rp, n, int(anyhit), threads, prim.ctypes.data_as(C.POINTER(C.c_uint32)),
                            t.ctypes.data_as(C.POINTER(C.c_float)), b1.ctypes.data_as(C.POINTER(C.c_float)),
                            b2.ctypes.data_as(C.POINTER(C.c_float)))
        return (prim.astype(bool) if anyhit else prim), t, b1, b2

    def spectrum_eval(self, spectrum_index: int, lambdas: np.ndarray) -> np.ndarray:
        lam, lp = _f(lambdas.reshape(-1, 16))
        out = np.zeros_like(lam)
        lib().ora_spectrum_eval(self.h, self.spectrum_ids[spectrum_index], lp, len(lam),
                                out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def medium_query(self, mode: int, rays: np.ndarray, lambdas: np.ndarray, sel: np.ndarray,
                     vals: np.ndarray) -> np.ndarray:
        """DensityGridMediumDistribution interact (0) / evaluateTransmittance
        (1) / evaluateExtinctionCoefficient (2) with the free-path sampler
        replaying `vals` (see ora_medium_query in ref_driver.cpp for the
        layouts); returns n x 24 floats."""
        r, rp = _f(rays.reshape(-1, 8))
        lam, lp = _f(lambdas.reshape(-1, 16))
        sl = np.ascontiguousarray(sel, np.int32)
        v, vp = _u(vals.reshape(len(r), -1))
        out = np.zeros((len(r), 24), np.float32)
        rc = lib().ora_medium_query(self.h, int(mode), len(r), rp, lp, sl.ctypes.data_as(C.POINTER(C.c_int)), vp,
                                    v.shape[1], out.ctypes.data_as(C.POINTER(C.c_float)))
        if rc != 0:
            raise RuntimeError("scene has no medium")
        return out


BSDF_KINDS = {"lambert": 0, "specular_brdf": 1, "specular_bsdf": 2, "ggx_brdf": 3, "ggx_bsdf": 4}


def bsdf_query(kind: str, spec0, spec1=None, spec2=None, ax=0.0, ay=0.0, queries=None) -> np.ndarray:
    """Evaluates a reference BSDF (see ora_bsdf_query in ref_driver.cpp for
    the 16-float query and 40-float result layouts)."""
    s0, s0p = _f(spec0)
    s1, s1p = _f(spec1 if spec1 is not None else spec0)
    s2, s2p = _f(spec2 if spec2 is not None else spec0)
    q, qp = _f(queries)
    out = np.zeros((len(q), 40), np.float32)
    rc = lib().ora_bsdf_query(BSDF_KINDS[kind], s0p, s1p, s2p, ax, ay, qp, len(q),
                              out.ctypes.data_as(C.POINTER(C.c_float)))
    if rc != 0:
        raise ValueError(kind)
    return out


def film_bmp(film: np.ndarray, scale: float, sensitivity: float, path: str) -> None:
    """Writes the film (h, w, 16) as a BMP with the reference's
    ImageSensor::saveImage."""
    f, fp = _f(np.ascontiguousarray(film, np.float32).reshape(-1))
    h, w = film.shape[:2]
    lib().ora_film_bmp(fp, w, h, float(scale), float(sensitivity), path.encode())


def film_cmf():
    """(bins (48,), integral) of the reference's discretised CMF."""
    bins = np.zeros(48, np.float32)
    integ = np.zeros(1, np.float32)
    lib().ora_film_cmf(bins.ctypes.data_as(C.POINTER(C.c_float)), integ.ctypes.data_as(C.POINTER(C.c_float)))
    return bins, float(integ[0])
