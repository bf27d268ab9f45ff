"""The C++ shim behind the reference's renderer interface
(include/slrgpu_renderer.hpp), compiled against the reference's own libSLR
headers and exercised end to end.

tests/shim_app.cpp is an application that builds each scene through the
reference's node API and, with the same calls, through SLRGPU::SceneBuilder;
it then renders the reference's SLR::Scene through a const SLR::Renderer&
(libSLR/Core/renderer.h:15-19) bound to SLRGPU::PathTracingRenderer and its
volumetric and bidirectional variants, and reads the film back from the
camera's ImageSensor (ImageSensor.h:47-48).  The sensor must hold, bit for
bit, the film slrgpu_render returns for the same scene and settings."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from slr_gb300 import scenes

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "tests", "_build", "libshim_app.so")


@pytest.fixture(scope="module")
def shim_app(gpu_lib, oracle_lib):
    """Builds the test application (a few seconds of g++) and binds its
    app_* calls under the ora_* names oracle.RefScene drives."""
    gpu_lib.lib()
    oracle_lib.lib()
    src_inc = os.path.join(ROOT, "oracle", "_ref", "src", "libSLR")
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    gpu_dir = os.path.join(ROOT, "slr_gb300", "lib")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-std=gnu++14", "-O2", "-fPIC", "-shared", "-w", "-include", "cstring", "-include", "cmath",
           f"-I{src_inc}", f"-I{os.path.join(ROOT, 'include')}", os.path.join(ROOT, "tests", "shim_app.cpp"),
           f"-L{ref_dir}", "-lslr_ref", f"-L{gpu_dir}", "-lslrgpu", f"-Wl,-rpath,{ref_dir}", f"-Wl,-rpath,{gpu_dir}",
           "-o", OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    L = C.CDLL(OUT)
    P, I, F = C.c_void_p, C.c_int, C.c_float
    fp, up = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
    sig = {
        "scene_new": (P, []), "scene_free": (None, [P]),
        "spectrum_rgb": (I, [P, I, F, F, F]), "spectrum_regular": (I, [P, F, F, fp, I]),
        "spectrum_irregular": (I, [P, fp, fp, I]), "material_matte": (I, [P, I]),
        "material_specular_reflection": (I, [P, I, I, I]), "material_specular_scattering": (I, [P, I, I, I]),
        "material_microfacet_reflection": (I, [P, I, I, F, F]),
        "material_microfacet_scattering": (I, [P, I, I, F, F]), "material_emitter": (I, [P, I, I]),
        "mesh": (I, [P, fp, fp, fp, fp, I, up, I, I]), "env_ibl": (I, [P, C.POINTER(C.c_uint16), I, I, F]),
        "medium_density_grid": (I, [P, fp, fp, I, I, fp, I, I, I, F]),
        "camera_perspective": (I, [P, fp, F, F, F, F, F, F]), "camera_equirect": (I, [P, fp, F, F, F]),
        "build": (I, [P]), "build_reference_only": (I, [P]), "device_scene": (C.c_uint64, [P]),
        "render": (I, [P, I, I, I, I, I, I, fp, C.POINTER(C.c_ulonglong)]),
    }

    class App:
        pass

    app = App()
    for name, (res, args) in sig.items():
        fn = getattr(L, "app_" + name)
        fn.restype, fn.argtypes = res, args
        setattr(app, "ora_" + name, fn)
        setattr(app, name, fn)
    return app


def _scene(oracle_lib, app, desc):
    s = oracle_lib.RefScene(desc, library=app)
    assert min(s.spectrum_ids) >= 0, "the two builders handed out different ids"
    return s


KINDS = {"pt": 0, "vol": 1, "bpt": 2, "vbpt": 3}


def _desc(name):
    if name == "box_irregular":
        d = scenes.box_scene(24, 16)
        # the back wall's reflectance as an irregular (tabulated) spectrum
        wl = np.array([380.0, 450.0, 520.0, 600.0, 700.0, 780.0], np.float32)
        v = np.array([0.2, 0.5, 0.8, 0.6, 0.4, 0.3], np.float32)
        d.meshes[2].material = d.material("matte", (d.spectrum_irregular(wl, v),))
        return d
    if name == "ggx_ibl":
        return scenes.heightfield_scene(grid=24, spheres=5, sphere_freq=3, env_size=(64, 32), width=20, height=20)
    if name == "medium":
        return scenes.medium_box_scene(16, 16, grid=16)
    if name == "equirect":
        from tests.image_cases import camera_override
        d = scenes.box_scene(32, 16)
        d.camera = camera_override("equirect", 32, 16)
        return d
    return scenes.box_scene(20, 12)


@pytest.mark.parametrize("name,kind", [("box_irregular", "pt"), ("ggx_ibl", "pt"), ("medium", "vol"),
                                       ("equirect", "pt"), ("box", "bpt"), ("medium", "vbpt")])
def test_renderer_interface_writes_the_sensor(gpu_lib, oracle_lib, shim_app, name, kind):
    desc = _desc(name)
    w, h = (32, 16) if name == "equirect" else (24, 16) if name == "box_irregular" else \
        (20, 20) if name == "ggx_ibl" else (16, 16) if name == "medium" else (20, 12)
    spp, depth, seed = 4, 8, 17
    s = _scene(oracle_lib, shim_app, desc)
    film = np.zeros((h, w, 16), np.float32)
    dropped = C.c_ulonglong(0)
    rc = shim_app.render(s.h, KINDS[kind], spp, depth, w, h, seed, film.ctypes.data_as(C.POINTER(C.c_float)),
                         C.byref(dropped))
    assert rc == 0, gpu_lib.lib().slrgpu_last_error()
    direct, st = gpu_lib.Scene(desc).render(w, h, spp, depth, seed=seed, volumetric=kind in ("vol", "vbpt"),
                                            bpt=kind in ("bpt", "vbpt"))
    assert film.sum() > 0
    if kind in ("bpt", "vbpt"):
        # the bidirectional splat film takes float atomics: reproducible to
        # rounding, not bit for bit
        np.testing.assert_allclose(film, direct, rtol=1e-4, atol=1e-6)
    else:
        np.testing.assert_array_equal(film.view(np.uint32), direct.view(np.uint32))
        assert dropped.value == st.dropped_samples


def test_unregistered_scene_is_an_error(gpu_lib, oracle_lib, shim_app):
    """An SLR::Scene whose device scene was never committed is not in the
    shim's registry: render() throws, and the application sees the error."""
    s = oracle_lib.RefScene(scenes.box_scene(8, 8), build=False, library=shim_app)
    assert shim_app.build_reference_only(s.h) == 0
    film = np.zeros((8, 8, 16), np.float32)
    rc = shim_app.render(s.h, 0, 1, 1, 8, 8, 0, film.ctypes.data_as(C.POINTER(C.c_float)), None)
    assert rc == -101
