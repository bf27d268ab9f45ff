"""Python mirror of the reference renderer's interface over the C ABI.

The classes follow SLR's names and argument meaning so that code written
against the reference reads the same:

* :class:`RenderSettings` - the typed settings map of libSLR/Core/RenderSettings.h:15-43
  (NumThreads, ImageWidth, ImageHeight, TimeStart, TimeEnd, Brightness, RNGSeed).
* :class:`Scene` - a committed scene (libSLR/Scene/Scene.h:17-52) built from a
  :class:`~slr_gb300.scene_desc.SceneDesc`.
* :class:`PathTracingRenderer` / :class:`VolumetricPathTracingRenderer` -
  ``render(scene, settings)`` like SLR::Renderer::render
  (libSLR/Core/renderer.h:15-19), returning the 16-bin film that
  ImageSensor::pixel(x, y) exposes (per pixel the sum over all samples).

Everything runs in the CUDA library ``slr_gb300/lib/libslrgpu.so``; there is
no CPU fallback: the classes raise when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
import re
from pathlib import Path

import numpy as np

from .scene_desc import SceneDesc

PKG = Path(__file__).resolve().parent
# SLRGPU_LIB_VARIANT=w8 loads the build with 8-wide BVH nodes
# (slr_gb300/build.py); the default is the tuned build.
_VARIANT = os.environ.get("SLRGPU_LIB_VARIANT", "")
LIB_PATH = PKG / "lib" / (f"libslrgpu_{_VARIANT}.so" if _VARIANT else "libslrgpu.so")
HEADER = PKG.parent / "include" / "slrgpu.h"

_lib = None


class SlrGpuError(RuntimeError):
    """A negative status of the C ABI; ``code`` holds it."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


ERR_TIMEOUT, ERR_CANCELLED = -7, -9
FAULT_SERVER_FILM_ALLOC, FAULT_SERVER_WAVE_LAUNCH = 0, 1


class BvhStats(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("num_fragments", C.c_uint32), ("depth", C.c_uint32),
                ("num_binary_nodes", C.c_uint32), ("num_wide_nodes", C.c_uint32), ("width", C.c_uint32),
                ("sah_cost", C.c_float), ("build_seconds", C.c_float)]


class Settings(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32), ("max_depth", C.c_uint32),
                ("seed", C.c_uint32), ("volumetric", C.c_uint32), ("samples_per_wave", C.c_uint32),
                ("flags", C.c_uint32), ("sample_base", C.c_uint32)]


KERNEL_CLASSES = ["raygen", "extend", "shade", "shadow", "accumulate"]
FLAG_PROFILE_KERNELS = 1
FLAG_WATERTIGHT = 2
FLAG_BPT = 4


class RenderStats(C.Structure):
    _fields_ = [("seconds", C.c_double), ("kernel_seconds", C.c_double), ("path_samples", C.c_uint64),
                ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("dropped_samples", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("kernel_ms", C.c_double * 8), ("kernel_count", C.c_uint64 * 8)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("kernel_ms", "kernel_count")}
        d["kernel_ms"] = {n: self.kernel_ms[i] for i, n in enumerate(KERNEL_CLASSES)}
        d["kernel_count"] = {n: self.kernel_count[i] for i, n in enumerate(KERNEL_CLASSES)}
        return d


class ServerConfig(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("slots", C.c_uint32), ("paths_per_slot", C.c_uint32),
                ("max_depth", C.c_uint32), ("hbm_budget_bytes", C.c_uint64)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("spp_done", C.c_uint32), ("submit_seconds", C.c_double),
                ("start_seconds", C.c_double), ("done_seconds", C.c_double), ("path_samples", C.c_uint64),
                ("dropped_samples", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [("requests_done", C.c_uint64), ("path_samples_done", C.c_uint64), ("waves", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("bytes_in_use", C.c_uint64), ("queued", C.c_uint32),
                ("active", C.c_uint32), ("first_start_seconds", C.c_double), ("last_done_seconds", C.c_double),
                ("mixed_scene_waves", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SERVER_PLAIN, SERVER_BATCHED = 0, 1
REQUEST_QUEUED, REQUEST_RUNNING, REQUEST_DONE = 0, 1, 2


def header_symbols() -> list[str]:
    """Every function the C ABI header declares."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|void|uint64_t)\s+(slrgpu_\w+)\s*\(", text, re.M)))


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.is_file():
            raise SlrGpuError(f"CUDA extension not built: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(str(LIB_PATH))
        H, I, U, F, P = C.c_uint64, C.c_int, C.c_uint32, C.c_float, C.c_void_p
        fp, up, ip, hp = C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_int), C.POINTER(C.c_uint64)
        u16p = C.POINTER(C.c_uint16)
        sig = {
            "slrgpu_last_error": (C.c_char_p, []),
            "slrgpu_version": (I, []),
            "slrgpu_context_create": (I, [I, hp]),
            "slrgpu_context_destroy": (I, [H]),
            "slrgpu_scene_create": (I, [H, hp]),
            "slrgpu_scene_destroy": (I, [H]),
            "slrgpu_spectrum_rgb": (I, [H, I, F, F, F, ip]),
            "slrgpu_spectrum_regular": (I, [H, F, F, fp, U, ip]),
            "slrgpu_spectrum_irregular": (I, [H, fp, fp, U, ip]),
            "slrgpu_material_matte": (I, [H, I, ip]),
            "slrgpu_material_specular_reflection": (I, [H, I, I, I, ip]),
            "slrgpu_material_specular_scattering": (I, [H, I, I, I, ip]),
            "slrgpu_material_microfacet_reflection": (I, [H, I, I, F, F, ip]),
            "slrgpu_material_microfacet_scattering": (I, [H, I, I, F, F, ip]),
            "slrgpu_material_emitter": (I, [H, I, I, ip]),
            "slrgpu_scene_add_mesh": (I, [H, fp, fp, fp, fp, U, up, U, I]),
            "slrgpu_environment_ibl": (I, [H, u16p, U, U, F]),
            "slrgpu_medium_density_grid": (I, [H, fp, fp, I, I, fp, U, U, U, F]),
            "slrgpu_medium_density_grid_file": (I, [H, C.c_char_p, fp, fp, I, I, F]),
            "slrgpu_camera_perspective": (I, [H, fp, F, F, F, F, F, F]),
            "slrgpu_camera_equirect": (I, [H, fp, F, F, F]),
            "slrgpu_scene_commit": (I, [H, C.POINTER(BvhStats)]),
            "slrgpu_scene_build_host": (I, [H, C.POINTER(BvhStats)]),
            "slrgpu_render": (I, [H, C.POINTER(Settings), P, I, C.POINTER(RenderStats)]),
            "slrgpu_render_continue": (I, [H, C.POINTER(Settings), fp, fp, C.POINTER(RenderStats)]),
            "slrgpu_render_replay": (I, [H, C.POINTER(Settings), fp, fp, C.POINTER(RenderStats)]),
            "slrgpu_context_queue_counts": (I, [H, up, U, up]),
            "slrgpu_trace": (I, [H, P, U, I, P, P, P, P, P]),
            "slrgpu_scene_sbvh_dump": (I, [H, fp, up, up]),
            "slrgpu_spectrum_evaluate": (I, [H, I, fp, U, fp]),
            "slrgpu_environment_tables": (I, [H, up, up, fp, fp, fp, fp, fp]),
            "slrgpu_bsdf_query": (I, [I, fp, fp, fp, F, F, fp, U, fp]),
            "slrgpu_scene_reupload": (I, [H, C.POINTER(C.c_uint64)]),
            "slrgpu_render_noalloc": (I, [H, C.POINTER(Settings), P, P]),
            "slrgpu_render_noalloc_scratch_bytes": (C.c_uint64, []),
            "slrgpu_medium_query": (I, [H, I, U, fp, fp, ip, up, U, fp]),
            "slrgpu_server_create": (I, [H, C.POINTER(ServerConfig), hp]),
            "slrgpu_server_destroy": (I, [H]),
            "slrgpu_server_submit": (I, [H, H, C.POINTER(Settings), hp]),
            "slrgpu_server_poll": (I, [H, C.c_uint64, C.POINTER(RequestInfo)]),
            "slrgpu_server_wait": (I, [H, C.c_uint64, fp, C.POINTER(RequestInfo), C.c_double]),
            "slrgpu_server_get_stats": (I, [H, C.POINTER(ServerStats)]),
            "slrgpu_server_cancel": (I, [H, C.c_uint64]),
            "slrgpu_server_set_deadline": (I, [H, C.c_uint64, C.c_double]),
            "slrgpu_debug_inject_fault": (I, [I, U]),
            "slrgpu_film_to_bmp": (I, [fp, U, U, I, F, F, C.POINTER(C.c_uint8), C.c_char_p]),
            "slrgpu_film_cmf": (I, [fp, fp]),
            "slrgpu_scene_alias_tables": (I, [H, up, fp, up, fp, up, fp, up]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        raise SlrGpuError(f"slrgpu error {rc}: {lib().slrgpu_last_error().decode()}", rc)


def inject_fault(site: int, count: int) -> None:
    """Host-side fault injection (slrgpu_debug_inject_fault): the next
    `count` film allocations (FAULT_SERVER_FILM_ALLOC) or wave launches
    (FAULT_SERVER_WAVE_LAUNCH) of any server fail; 0 clears the site."""
    check(lib().slrgpu_debug_inject_fault(site, count))


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class RenderSettingItem(enum.Enum):
    NumThreads = 0
    ImageWidth = 1
    ImageHeight = 2
    TimeStart = 3
    TimeEnd = 4
    Brightness = 5
    RNGSeed = 6


class RenderSettings:
    """Typed key/value settings (libSLR/Core/RenderSettings.h:24-43)."""

    def __init__(self, **items):
        self._items = {}
        for k, v in items.items():
            self.addItem(RenderSettingItem[k], v)

    def addItem(self, item: RenderSettingItem, value) -> None:
        self._items[item] = value

    def get(self, item: RenderSettingItem, default=None):
        return self._items.get(item, default)


class Context:
    """One GPU (device index); owns path-state and film buffers."""

    def __init__(self, device: int = 0):
        h = C.c_uint64()
        check(lib().slrgpu_context_create(device, C.byref(h)))
        self.handle = h.value

    def queue_counts(self) -> np.ndarray:
        """(rows, 11) queue counters of the last path-tracer wave rendered on
        this context (slrgpu_context_queue_counts)."""
        cap = 11 * 4096
        out = np.zeros(cap, np.uint32)
        rows = C.c_uint32()
        check(lib().slrgpu_context_queue_counts(self.handle, _up(out), cap, C.byref(rows)))
        return out[:11 * rows.value].reshape(rows.value, 11)

    def close(self):
        if getattr(self, "handle", 0):
            lib().slrgpu_context_destroy(self.handle)
            self.handle = 0


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class Scene:
    """A scene on the device built from a SceneDesc (tee of the reference's
    node-API construction: same spectra, materials, meshes, environment,
    camera)."""

    def __init__(self, desc: SceneDesc, context: Context | None = None, commit: bool = True,
                 host_only: bool = False):
        L = lib()
        self.desc = desc
        self.context = None if host_only else (context or default_context())
        h = C.c_uint64()
        check(L.slrgpu_scene_create(0 if host_only else self.context.handle, C.byref(h)))
        self.handle = h.value
        self._keep = []
        sid = []
        out = C.c_int()
        for sp in desc.spectra:
            if sp.kind == "rgb":
                check(L.slrgpu_spectrum_rgb(self.handle, sp.sp_type, *sp.rgb, C.byref(out)))
            elif sp.kind == "regular":
                v = np.ascontiguousarray(sp.values, np.float32)
                check(L.slrgpu_spectrum_regular(self.handle, sp.min_wl, sp.max_wl, _fp(v), len(v), C.byref(out)))
            else:
                w = np.ascontiguousarray(sp.wavelengths, np.float32)
                v = np.ascontiguousarray(sp.values, np.float32)
                check(L.slrgpu_spectrum_irregular(self.handle, _fp(w), _fp(v), len(v), C.byref(out)))
            sid.append(out.value)
        mid = []
        for m in desc.materials:
            s = [sid[i] for i in m.spectra]
            if m.kind == "matte":
                check(L.slrgpu_material_matte(self.handle, s[0], C.byref(out)))
            elif m.kind == "specular_reflection":
                check(L.slrgpu_material_specular_reflection(self.handle, *s, C.byref(out)))
            elif m.kind == "specular_scattering":
                check(L.slrgpu_material_specular_scattering(self.handle, *s, C.byref(out)))
            elif m.kind == "microfacet_reflection":
                check(L.slrgpu_material_microfacet_reflection(self.handle, s[0], s[1], m.alpha_x, m.alpha_y,
                                                              C.byref(out)))
            elif m.kind == "microfacet_scattering":
                check(L.slrgpu_material_microfacet_scattering(self.handle, s[0], s[1], m.alpha_x, m.alpha_y,
                                                              C.byref(out)))
            elif m.kind == "emitter":
                check(L.slrgpu_material_emitter(self.handle, mid[m.base], s[0], C.byref(out)))
            else:
                raise ValueError(m.kind)
            mid.append(out.value)
        for mesh in desc.meshes:
            p = np.ascontiguousarray(mesh.positions, np.float32)
            n = np.ascontiguousarray(mesh.normals, np.float32)
            t = np.ascontiguousarray(mesh.tangents, np.float32)
            uv = np.ascontiguousarray(mesh.uvs, np.float32)
            idx = np.ascontiguousarray(mesh.indices, np.uint32)
            check(L.slrgpu_scene_add_mesh(self.handle, _fp(p), _fp(n), _fp(t), _fp(uv), len(p), _up(idx), len(idx),
                                          mid[mesh.material]))
        if desc.environment is not None:
            img = np.ascontiguousarray(desc.environment.rgba_half, np.float16).view(np.uint16)
            check(L.slrgpu_environment_ibl(self.handle, img.ctypes.data_as(C.POINTER(C.c_uint16)), img.shape[1],
                                           img.shape[0], desc.environment.scale))
        if desc.medium is not None:
            md = desc.medium
            bmin = np.asarray(md.bounds_min, np.float32)
            bmax = np.asarray(md.bounds_max, np.float32)
            dens = np.ascontiguousarray(md.density, np.float32)
            nz, ny, nx = dens.shape
            check(L.slrgpu_medium_density_grid(self.handle, _fp(bmin), _fp(bmax), sid[md.sigma_s], sid[md.sigma_e],
                                               _fp(dens), nx, ny, nz, md.hg_g))
        cam = desc.camera
        if cam is not None:
            m = np.ascontiguousarray(cam.cam_to_world, np.float32)
            if cam.kind == "perspective":
                check(L.slrgpu_camera_perspective(self.handle, _fp(m), cam.sensitivity, cam.aspect, cam.fov_y,
                                                  cam.lens_radius, cam.img_plane_dist, cam.obj_plane_dist))
            else:
                check(L.slrgpu_camera_equirect(self.handle, _fp(m), cam.sensitivity, cam.phi_angle, cam.theta_angle))
        self.spectrum_ids = sid
        self.material_ids = mid
        self.bvh_stats = None
        if host_only:
            st = BvhStats()
            check(L.slrgpu_scene_build_host(self.handle, C.byref(st)))
            self.bvh_stats = st
        elif commit:
            self.commit()

    def commit(self) -> BvhStats:
        st = BvhStats()
        check(lib().slrgpu_scene_commit(self.handle, C.byref(st)))
        self.bvh_stats = st
        return st

    def close(self):
        if getattr(self, "handle", 0):
            lib().slrgpu_scene_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- rendering / queries ------------------------------------------------
    def reupload(self) -> int:
        """Copies the scene's device arrays again from their pinned host
        mirrors; returns the bytes copied."""
        b = C.c_uint64()
        check(lib().slrgpu_scene_reupload(self.handle, C.byref(b)))
        return b.value

    def render(self, width: int, height: int, spp: int, max_depth: int, seed: int = 0, volumetric: bool = False,
               samples_per_wave: int = 0, film=None, flags: int = 0, sample_base: int = 0, bpt: bool = False):
        """Returns (film (h, w, 16) float32 sum over samples, RenderStats).
        ``film`` may be a preallocated host numpy array or a CUDA tensor;
        samples [sample_base, sample_base + spp) are rendered.  ``bpt``:
        bidirectional path tracing (max_depth then caps each subpath)."""
        if bpt:
            flags |= FLAG_BPT
        s = Settings(width, height, spp, max_depth, seed, int(volumetric), samples_per_wave, flags, sample_base)
        st = RenderStats()
        on_device = 0
        if film is None:
            film = np.zeros((height, width, 16), np.float32)
            ptr = film.ctypes.data
        elif isinstance(film, np.ndarray):
            ptr = film.ctypes.data
        else:  # torch CUDA tensor
            on_device = 1
            ptr = film.data_ptr()
        check(lib().slrgpu_render(self.handle, C.byref(s), C.c_void_p(ptr), on_device, C.byref(st)))
        return film, st

    def render_continue(self, state: "FilmCheckpoint", spp: int, flags: int = 0):
        """Renders the next `spp` samples of a checkpointed film
        (slrgpu_render_continue) and advances the checkpoint; returns
        (film, RenderStats).  Rendering a frame over several calls, with the
        checkpoint saved and loaded in between, gives the one-call film bit
        for bit."""
        c = state
        s = Settings(c.width, c.height, spp, c.max_depth, c.seed, int(c.volumetric), 0, flags, c.next_sample)
        st = RenderStats()
        film = np.zeros((c.height, c.width, 16), np.float32)
        check(lib().slrgpu_render_continue(self.handle, C.byref(s), _fp(c.state), _fp(film), C.byref(st)))
        c.next_sample += spp
        c.dropped += st.dropped_samples
        return film, st

    def render_replay(self, width: int, height: int, max_depth: int, tapes: np.ndarray):
        """One sample per pixel in which the path of grid position i draws
        tapes[i] (256 uniforms each, tile-padded grid, row-major) instead of
        its own random numbers (slrgpu_render_replay).  Returns (film,
        RenderStats)."""
        t = np.ascontiguousarray(tapes, np.float32)
        s = Settings(width, height, 1, max_depth, 0, 0, 0, 0, 0)
        st = RenderStats()
        film = np.zeros((height, width, 16), np.float32)
        check(lib().slrgpu_render_replay(self.handle, C.byref(s), _fp(t), _fp(film), C.byref(st)))
        return film, st

    def trace(self, rays_dev, any_hit: bool = False, watertight: bool = False):
        """rays_dev: torch CUDA float32 tensor (n, 8).  Returns torch tensors
        (prim, t, b1, b2) on the same device (any hit: prim only); watertight
        selects the watertight triangle test instead of the reference's."""
        import torch
        n = rays_dev.shape[0]
        prim = torch.empty(n, dtype=torch.int32, device=rays_dev.device)
        if any_hit:
            t = b1 = b2 = None
            ptrs = [None, None, None]
        else:
            t = torch.empty(n, dtype=torch.float32, device=rays_dev.device)
            b1 = torch.empty_like(t)
            b2 = torch.empty_like(t)
            ptrs = [t.data_ptr(), b1.data_ptr(), b2.data_ptr()]
        stream = torch.cuda.current_stream(rays_dev.device).cuda_stream
        check(lib().slrgpu_trace(self.handle, C.c_void_p(rays_dev.data_ptr()), n, int(any_hit) | (2 * int(watertight)),
                                 C.c_void_p(prim.data_ptr()), *(C.c_void_p(p) if p else None for p in ptrs),
                                 C.c_void_p(stream)))
        return prim, t, b1, b2

    # -- host diagnostics -------------------------------------------------
    def sbvh_dump(self):
        st = self.bvh_stats
        boxes = np.zeros((st.num_binary_nodes, 6), np.float32)
        words = np.zeros((st.num_binary_nodes, 5), np.uint32)
        leaves = np.zeros(st.num_fragments, np.uint32)
        check(lib().slrgpu_scene_sbvh_dump(self.handle, _fp(boxes), _up(words), _up(leaves)))
        return boxes, words, leaves

    def spectrum_evaluate(self, spectrum_index: int, lambdas: np.ndarray) -> np.ndarray:
        lam = np.ascontiguousarray(lambdas, np.float32).reshape(-1, 16)
        out = np.zeros_like(lam)
        check(lib().slrgpu_spectrum_evaluate(self.handle, self.spectrum_ids[spectrum_index], _fp(lam), len(lam),
                                             _fp(out)))
        return out

    def medium_query(self, mode: int, rays: np.ndarray, lambdas: np.ndarray, sel: np.ndarray,
                     vals: np.ndarray) -> np.ndarray:
        """GPU medium queries with replayed uniforms (slrgpu_medium_query):
        mode 0 free-path sampling, 1 transmittance, 2 extinction coefficient;
        returns n x 24 floats."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        lam = np.ascontiguousarray(lambdas, np.float32).reshape(-1, 16)
        sl = np.ascontiguousarray(sel, np.int32)
        v = np.ascontiguousarray(vals, np.uint32).reshape(len(r), -1)
        out = np.zeros((len(r), 24), np.float32)
        check(lib().slrgpu_medium_query(self.handle, int(mode), len(r), _fp(r), _fp(lam),
                                        sl.ctypes.data_as(C.POINTER(C.c_int)), _up(v), v.shape[1], _fp(out)))
        return out

    def alias_tables(self):
        """Alias tables of the light and environment sampling (host build):
        dict of (prob, alias) pairs for 'lights', 'top' (rows), 'rows'."""
        n = C.c_uint32()
        check(lib().slrgpu_scene_alias_tables(self.handle, C.byref(n), None, None, None, None, None, None))
        out = {}
        lp, la = np.zeros(n.value, np.float32), np.zeros(n.value, np.uint32)
        args = [_fp(lp), _up(la)]
        if self.desc.environment is not None:
            h, w = self.desc.environment.rgba_half.shape[:2]
            mw, mh = w // 4, h // 4
            tp, ta = np.zeros(mh, np.float32), np.zeros(mh, np.uint32)
            rp, ra = np.zeros((mh, mw), np.float32), np.zeros((mh, mw), np.uint32)
            args += [_fp(tp), _up(ta), _fp(rp), _up(ra)]
            out["top"], out["rows"] = (tp, ta), (rp, ra)
        else:
            args += [None, None, None, None]
        check(lib().slrgpu_scene_alias_tables(self.handle, None, *args))
        out["lights"] = (lp, la)
        return out

    def environment_tables(self):
        env = self.desc.environment
        h, w = env.rgba_half.shape[:2]
        mw, mh = w // 4, h // 4
        row_pdf = np.zeros((mh, mw), np.float32)
        row_cdf = np.zeros((mh, mw + 1), np.float32)
        top_pdf = np.zeros(mh, np.float32)
        top_cdf = np.zeros(mh + 1, np.float32)
        texels = np.zeros((h, w, 4), np.float32)
        a, b = C.c_uint32(), C.c_uint32()
        check(lib().slrgpu_environment_tables(self.handle, C.byref(a), C.byref(b), _fp(row_pdf), _fp(row_cdf),
                                              _fp(top_pdf), _fp(top_cdf), _fp(texels)))
        return {"row_pdf": row_pdf, "row_cdf": row_cdf, "top_pdf": top_pdf, "top_cdf": top_cdf, "texels": texels}


BSDF_KINDS = {"lambert": 0, "specular_brdf": 1, "specular_bsdf": 2, "ggx_brdf": 3, "ggx_bsdf": 4}


def bsdf_query(kind: str, spec0, spec1=None, spec2=None, ax=0.0, ay=0.0, queries=None) -> np.ndarray:
    """Evaluates a BSDF on the GPU at fixed (query, sample) tuples; the
    16-float query and 40-float result layouts of slrgpu_bsdf_query."""
    s0 = np.ascontiguousarray(spec0, np.float32)
    s1 = np.ascontiguousarray(spec1 if spec1 is not None else spec0, np.float32)
    s2 = np.ascontiguousarray(spec2 if spec2 is not None else spec0, np.float32)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 16)
    out = np.zeros((len(q), 40), np.float32)
    check(lib().slrgpu_bsdf_query(BSDF_KINDS[kind], _fp(s0), _fp(s1), _fp(s2), ax, ay, _fp(q), len(q), _fp(out)))
    return out


class FilmCheckpoint:
    """A resumable render: the settings, the next sample index, the dropped
    sample count and the compensated film sums (2 x 16 x height x width
    floats), saved to and loaded from an .npz file."""

    def __init__(self, width: int, height: int, max_depth: int, seed: int = 0, volumetric: bool = False):
        self.width, self.height, self.max_depth = int(width), int(height), int(max_depth)
        self.seed, self.volumetric = int(seed), bool(volumetric)
        self.next_sample = 0
        self.dropped = 0
        self.state = np.zeros(2 * 16 * self.width * self.height, np.float32)

    def film(self) -> np.ndarray:
        """The film (height, width, 16) of the samples rendered so far."""
        return np.ascontiguousarray(self.state[:16 * self.width * self.height].reshape(16, self.height, self.width)
                                    .transpose(1, 2, 0))

    def save(self, path: str) -> None:
        np.savez(path, state=self.state, meta=np.array([self.width, self.height, self.max_depth, self.seed,
                                                         int(self.volumetric), self.next_sample, self.dropped],
                                                        np.int64))

    @classmethod
    def load(cls, path: str) -> "FilmCheckpoint":
        d = np.load(path)
        w, h, depth, seed, vol, nxt, dropped = (int(v) for v in d["meta"])
        c = cls(w, h, depth, seed, bool(vol))
        c.next_sample, c.dropped = nxt, dropped
        state = np.ascontiguousarray(d["state"], np.float32)
        if state.shape != c.state.shape:
            raise ValueError("checkpoint state does not match its settings")
        c.state = state
        return c


class Server:
    """Serving loop with continuous batching (slrgpu_server_*): submit render
    requests of any committed scene of the context; wait() returns the film,
    bit-identical to Scene.render with the same settings."""

    def __init__(self, context: Context | None = None, mode: int = SERVER_BATCHED, slots: int = 0,
                 paths_per_slot: int = 0, max_depth: int = 0, hbm_budget_bytes: int = 0):
        self.context = context or default_context()
        cfg = ServerConfig(mode, slots, paths_per_slot, max_depth, hbm_budget_bytes)
        h = C.c_uint64()
        check(lib().slrgpu_server_create(self.context.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value
        self._shapes = {}

    def submit(self, scene: "Scene", width: int, height: int, spp: int, max_depth: int, seed: int = 0,
               volumetric: bool = False) -> int:
        s = Settings(width, height, spp, max_depth, seed & 0xffffffff, int(volumetric), 0, 0)
        rid = C.c_uint64()
        check(lib().slrgpu_server_submit(self.handle, scene.handle, C.byref(s), C.byref(rid)))
        self._shapes[rid.value] = (height, width)
        return rid.value

    def poll(self, request: int) -> RequestInfo:
        info = RequestInfo()
        check(lib().slrgpu_server_poll(self.handle, request, C.byref(info)))
        return info

    def wait(self, request: int, timeout: float = -1.0):
        """Returns (film, RequestInfo); raises SlrGpuError with the request's
        status (e.g. ERR_CANCELLED, or ERR_TIMEOUT when `timeout` passes
        first, in which case the request stays queued or running)."""
        h, w = self._shapes[request]
        film = np.zeros((h, w, 16), np.float32)
        info = RequestInfo()
        rc = lib().slrgpu_server_wait(self.handle, request, _fp(film), C.byref(info), float(timeout))
        if rc != ERR_TIMEOUT:
            self._shapes.pop(request, None)
        check(rc)
        return film, info

    def cancel(self, request: int) -> None:
        check(lib().slrgpu_server_cancel(self.handle, request))

    def set_deadline(self, request: int, seconds: float) -> None:
        check(lib().slrgpu_server_set_deadline(self.handle, request, float(seconds)))

    def stats(self) -> ServerStats:
        st = ServerStats()
        check(lib().slrgpu_server_get_stats(self.handle, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "handle", 0):
            lib().slrgpu_server_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def film_to_bmp(film: np.ndarray, scale: float = 1.0, sensitivity: float = 1.0, path: str | None = None):
    """ImageSensor::saveImage on the GPU (slrgpu_film_to_bmp): returns the BMP
    pixel array (bottom-up BGR rows padded to 4 bytes) of an (h, w, 16) film
    and writes a BMP file when `path` is given."""
    f = np.ascontiguousarray(film, np.float32)
    h, w = f.shape[:2]
    row = 3 * w + w % 4
    px = np.zeros(row * h, np.uint8)
    check(lib().slrgpu_film_to_bmp(_fp(f), w, h, 0, float(scale), float(sensitivity),
                                   px.ctypes.data_as(C.POINTER(C.c_uint8)), path.encode() if path else None))
    return px.reshape(h, row)


def film_cmf():
    """(x, y, z bins of the colour matching functions (3, 16), y integral)."""
    bins = np.zeros(48, np.float32)
    integ = np.zeros(1, np.float32)
    check(lib().slrgpu_film_cmf(_fp(bins), _fp(integ)))
    return bins.reshape(3, 16), float(integ[0])


class PathTracingRenderer:
    """Drop-in for SLR::PTRenderer(spp) (libSLR/Renderer/PTRenderer.h:42-43)
    with the max-depth parameter the GPU path adds."""

    volumetric = False

    def __init__(self, spp: int, max_depth: int = 100):
        self.spp = int(spp)
        self.max_depth = int(max_depth)

    def render(self, scene: Scene, settings: RenderSettings):
        w = int(settings.get(RenderSettingItem.ImageWidth))
        h = int(settings.get(RenderSettingItem.ImageHeight))
        seed = int(settings.get(RenderSettingItem.RNGSeed, 0)) & 0xffffffff
        film, stats = scene.render(w, h, self.spp, self.max_depth, seed=seed, volumetric=self.volumetric)
        self.last_stats = stats
        return film


class BidirectionalPathTracingRenderer:
    """Drop-in for SLR::BPTRenderer(spp) (libSLR/Renderer/BPTRenderer.h:117-123);
    max_depth caps each subpath at that many vertices beyond its first (the
    reference ends subpaths by Russian roulette only)."""

    volumetric = False

    def __init__(self, spp: int, max_depth: int = 32):
        self.spp = int(spp)
        self.max_depth = int(max_depth)

    def render(self, scene: Scene, settings: RenderSettings):
        w = int(settings.get(RenderSettingItem.ImageWidth))
        h = int(settings.get(RenderSettingItem.ImageHeight))
        seed = int(settings.get(RenderSettingItem.RNGSeed, 0)) & 0xffffffff
        film, stats = scene.render(w, h, self.spp, self.max_depth, seed=seed, bpt=True, volumetric=self.volumetric)
        self.last_stats = stats
        return film


class VolumetricBidirectionalPathTracingRenderer(BidirectionalPathTracingRenderer):
    """Drop-in for SLR::VolumetricBPTRenderer(spp)
    (libSLR/Renderer/VolumetricBPTRenderer.h:121)."""

    volumetric = True


class VolumetricPathTracingRenderer(PathTracingRenderer):
    """Drop-in for SLR::VolumetricPTRenderer(spp)
    (libSLR/Renderer/VolumetricPTRenderer.h:43-44)."""

    volumetric = True
