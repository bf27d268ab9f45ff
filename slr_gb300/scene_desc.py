"""Plain-array scene description shared by the GPU renderer and its checkers.

A :class:`SceneDesc` is the data a caller hands to the renderer: spectra,
materials, triangle meshes (world-space vertices), an optional image-based
environment, an optional density-grid medium and a camera.  It mirrors the
inputs of the reference's node API (libSLR/Scene/TriangleMeshNode.h:17-73,
Scene/node.h:125-141, Scene/camera_nodes.h:16-54, Scene/medium_nodes.h:33-48)
so that the same description can be rendered by the GPU path and by the
reference.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

import numpy as np

# Spectrum types of the reference (libSLR/BasicTypes/spectrum_base.h:34-38).
REFLECTANCE, LIGHT_SOURCE, INDEX_OF_REFRACTION = 0, 1, 2


@dataclass
class Spectrum:
    kind: str                      # "rgb" | "regular" | "irregular"
    sp_type: int = REFLECTANCE     # for "rgb"
    rgb: tuple = (0.0, 0.0, 0.0)   # linear sRGB, for "rgb"
    min_wl: float = 360.0          # for "regular"
    max_wl: float = 830.0
    values: np.ndarray | None = None
    wavelengths: np.ndarray | None = None  # for "irregular"


@dataclass
class Material:
    kind: str   # matte | specular_reflection | specular_scattering |
                # microfacet_reflection | microfacet_scattering | emitter
    spectra: tuple = ()            # spectrum indices, meaning per kind (see api.py)
    alpha_x: float = 0.0
    alpha_y: float = 0.0
    base: int = -1                 # emitter: base (non-emitting) material index


@dataclass
class Mesh:
    positions: np.ndarray          # (nv, 3) float32
    normals: np.ndarray            # (nv, 3) float32
    tangents: np.ndarray           # (nv, 3) float32
    uvs: np.ndarray                # (nv, 2) float32
    indices: np.ndarray            # (nt, 3) uint32
    material: int


@dataclass
class Camera:
    kind: str                      # "perspective" | "equirect"
    cam_to_world: np.ndarray       # (4, 4) float32, row-major
    sensitivity: float = 1.0
    aspect: float = 1.0
    fov_y: float = 0.7
    lens_radius: float = 0.0
    img_plane_dist: float = 1.0
    obj_plane_dist: float = 1.0
    phi_angle: float = 2 * np.pi
    theta_angle: float = np.pi


@dataclass
class Environment:
    rgba_half: np.ndarray          # (h, w, 4) float16, linear RGBA
    scale: float = 1.0


@dataclass
class Medium:
    bounds_min: tuple
    bounds_max: tuple
    density: np.ndarray            # (nz, ny, nx) float32
    sigma_s: int                   # spectrum index (scattering coefficient base)
    sigma_e: int                   # spectrum index (extinction coefficient base)
    hg_g: float = 0.0


def write_density_grid(path: str, density: np.ndarray) -> None:
    """Writes a (nz, ny, nx) float32 grid in the reference's raw density-grid
    format: uint32 nx, ny, nz, then the slices (libSLRSceneGraph/API.cpp:966-989)."""
    d = np.ascontiguousarray(density, np.float32)
    nz, ny, nx = d.shape
    with open(path, "wb") as f:
        f.write(np.array([nx, ny, nz], np.uint32).tobytes())
        f.write(d.tobytes())


def read_density_grid(path: str) -> np.ndarray:
    """Reads the reference's raw density-grid format into a (nz, ny, nx) array."""
    raw = open(path, "rb").read()
    nx, ny, nz = np.frombuffer(raw[:12], np.uint32)
    d = np.frombuffer(raw[12:], np.float32)
    if d.size != int(nx) * int(ny) * int(nz):
        raise ValueError(f"malformed density grid file: {path}")
    return d.reshape(int(nz), int(ny), int(nx))


@dataclass
class SceneDesc:
    spectra: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    meshes: list = field(default_factory=list)
    camera: Camera | None = None
    environment: Environment | None = None
    medium: Medium | None = None

    # -- builders -------------------------------------------------------
    def spectrum_rgb(self, sp_type: int, r: float, g: float, b: float) -> int:
        self.spectra.append(Spectrum("rgb", sp_type=sp_type, rgb=(float(r), float(g), float(b))))
        return len(self.spectra) - 1

    def spectrum_regular(self, values, min_wl=360.0, max_wl=830.0) -> int:
        self.spectra.append(Spectrum("regular", min_wl=float(min_wl), max_wl=float(max_wl),
                                     values=np.ascontiguousarray(values, np.float32)))
        return len(self.spectra) - 1

    def spectrum_irregular(self, wavelengths, values) -> int:
        self.spectra.append(Spectrum("irregular", wavelengths=np.ascontiguousarray(wavelengths, np.float32),
                                     values=np.ascontiguousarray(values, np.float32)))
        return len(self.spectra) - 1

    def material(self, kind: str, spectra=(), alpha_x=0.0, alpha_y=0.0, base=-1) -> int:
        self.materials.append(Material(kind, tuple(int(s) for s in spectra), float(alpha_x), float(alpha_y), int(base)))
        return len(self.materials) - 1

    def mesh(self, positions, indices, material, normals=None, tangents=None, uvs=None) -> int:
        p = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        if normals is None or tangents is None:
            n, t = _flat_frames(p, idx)
            normals = n if normals is None else normals
            tangents = t if tangents is None else tangents
        if uvs is None:
            uvs = np.zeros((len(p), 2), np.float32)
        self.meshes.append(Mesh(p, np.ascontiguousarray(normals, np.float32).reshape(-1, 3),
                                np.ascontiguousarray(tangents, np.float32).reshape(-1, 3),
                                np.ascontiguousarray(uvs, np.float32).reshape(-1, 2), idx, int(material)))
        return len(self.meshes) - 1

    @property
    def num_triangles(self) -> int:
        return int(sum(len(m.indices) for m in self.meshes))

    def triangle_arrays(self):
        """Concatenated world-space triangles in the order the reference's
        Scene::build creates its surface objects (node order, then triangle
        order; TriangleMeshNode.cpp:77-99): returns (positions (nt,3,3))."""
        tris = [m.positions[m.indices] for m in self.meshes]
        return np.concatenate(tris, axis=0) if tris else np.zeros((0, 3, 3), np.float32)


def _flat_frames(p: np.ndarray, idx: np.ndarray):
    """Per-vertex normal/tangent for meshes given without them: the average
    of adjacent face normals, and a tangent orthogonal to it."""
    n = np.zeros_like(p, dtype=np.float64)
    tri = p[idx].astype(np.float64)
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    for k in range(3):
        np.add.at(n, idx[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1
    n /= ln
    a = np.where(np.abs(n[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t = a - (a * n).sum(1, keepdims=True) * n
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    return n.astype(np.float32), t.astype(np.float32)


def replace(desc: SceneDesc, **kw) -> SceneDesc:
    return dataclasses.replace(desc, **kw)
