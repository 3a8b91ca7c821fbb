"""Scene descriptions and the synthetic workloads.

A scene is built the way the reference's YAML factory builds one
(factory/creator/scene_creators.cpp:32-70): geometric primitives (quad,
cube, triangle mesh, optionally wrapped two-sided), a material per primitive
(Lambertian ``diffuse`` or ``disney``), an ordered light list (``directional``
and ``envmap`` with a constant texture) and a thin-lens camera.

``flatten`` turns a scene into the flat arrays the GPU library takes: the
triangles in the order the reference's PLOC aggregate gathers them
(core/aggregate/ploc_aggregate.cpp:259-285, primitives in order, triangles in
MeshView order), one flag word per triangle that selects the primitive's
PostIntersect rule, the world bounds the lights are fitted to
(core/scene/default_scene.cpp:32-48) and packed material and light records.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

F32 = np.float32

# Per-triangle PostIntersect rules (values shared with include/ajisai_gpu.h).
TRI_TWO_SIDED = 1    # TwoSided wrapper: normals flipped to face wr
TRI_NG_REVERSED = 2  # Cube: normal from the tuple order (k, j, i)
TRI_HAS_NORMALS = 4  # MeshGeo: interpolated per-vertex shading normals

MAT_DIFFUSE = 0
MAT_DISNEY = 1
MAT_MIRROR = 2
MAT_GLASS = 3
MAT_METAL = 4
MAT_PLASTIC = 5
MAT_NULL = 6
LIGHT_DIRECTIONAL = 0
LIGHT_ENV = 1


# --------------------------------------------------------------- materials --
@dataclass
class Material:
    """Constant-texture material; the record layout of ajg_material."""
    type: int
    base_color: Sequence[float] = (0.8, 0.8, 0.8)
    subsurface: float = 0.0
    metallic: float = 0.0
    specular: float = 0.0
    specular_tint: float = 0.0
    roughness: float = 0.0
    anisotropic: float = 0.0
    sheen: float = 0.0
    sheen_tint: float = 0.0
    clearcoat: float = 0.0
    clearcoat_gloss: float = 0.0
    # the ten parameter floats of the non-Disney types (None: the Disney
    # fields above)
    params: Optional[Sequence[float]] = None

    def pack(self) -> np.ndarray:
        r = np.zeros(16, F32)
        r[0] = self.type
        r[1:4] = self.base_color
        if self.params is not None:
            r[4:4 + len(self.params)] = self.params
        else:
            r[4:14] = [self.subsurface, self.metallic, self.specular,
                       self.specular_tint, self.roughness, self.anisotropic,
                       self.sheen, self.sheen_tint, self.clearcoat,
                       self.clearcoat_gloss]
        return r


def Diffuse(albedo) -> Material:
    """CreateDiffuse (core/material/diffuse.cpp:54-56)."""
    return Material(MAT_DIFFUSE, tuple(albedo))


def Disney(base_color, subsurface=0.0, metallic=0.0, specular=0.5,
           specular_tint=0.0, roughness=0.5, anisotropic=0.0, sheen=0.0,
           sheen_tint=0.0, clearcoat=0.0, clearcoat_gloss=0.0) -> Material:
    """CreateDisney (core/material/disney.cpp:541-553)."""
    return Material(MAT_DISNEY, tuple(base_color), subsurface, metallic,
                    specular, specular_tint, roughness, anisotropic, sheen,
                    sheen_tint, clearcoat, clearcoat_gloss)


def Mirror(kr) -> Material:
    """CreateMirror (core/material/mirror.cpp:100-102)."""
    return Material(MAT_MIRROR, tuple(np.broadcast_to(kr, 3)), params=())


def Glass(ior, color_reflection=1.0, color_refraction=1.0) -> Material:
    """CreateGlass (core/material/glass.cpp:160-165) with the YAML creator's
    defaults (material_creators.cpp:133-152): the refraction colour is
    stored as given; shading takes its square root."""
    return Material(MAT_GLASS, tuple(np.broadcast_to(color_reflection, 3)),
                    params=(*np.broadcast_to(color_refraction, 3), ior))


def Metal(color, k, eta, uroughness=0.1, vroughness=0.1) -> Material:
    """CreateMetal (core/material/metal.cpp:75-80): a GGX reflection with a
    coloured conductor Fresnel of (eta, k)."""
    return Material(MAT_METAL, tuple(np.broadcast_to(color, 3)),
                    params=(*np.broadcast_to(k, 3), *np.broadcast_to(eta, 3),
                            uroughness, vroughness))


def Plastic(albedo, ior=1.5, thickness=1.0, sigma_a=0.0) -> Material:
    """CreatePlastic (core/material/plastic.cpp:62-65) with the YAML
    creator's defaults (material_creators.cpp:44-52)."""
    return Material(MAT_PLASTIC, tuple(np.broadcast_to(albedo, 3)),
                    params=(ior, thickness, sigma_a))


def Null() -> Material:
    """CreateNull (core/material/null.cpp:74): rays pass straight through."""
    return Material(MAT_NULL, (0.0, 0.0, 0.0), params=())


# ------------------------------------------------------------------ lights --
@dataclass
class Light:
    type: int
    rgb: Sequence[float]
    direction: Sequence[float] = (0.0, 1.0, 0.0)  # toward the light
    angle: float = 0.0      # cone half-angle, radians
    scaler: float = 1.0
    rot: float = 0.0        # env map rotation, degrees

    def pack(self) -> np.ndarray:
        """ajg_light record: type, rgb, direction, cos(angle), scaler, rot."""
        r = np.zeros(12, F32)
        r[0] = self.type
        r[1:4] = self.rgb
        r[4:7] = self.direction
        r[7] = np.cos(F32(self.angle), dtype=F32)
        r[8] = self.scaler
        r[9] = self.rot
        return r

    def harness_pack(self) -> np.ndarray:
        r = self.pack()
        r[7] = self.angle
        return r


def DirectionalLight(direction, radiance, angle_deg: float = 0.0) -> Light:
    """CreateDirectionalLight (core/light/directional_light.cpp:98-101).
    ``direction`` points toward the light, as the YAML key does
    (factory/creator/light_creators.cpp:33)."""
    rad = float(F32(angle_deg) * F32(3.141592654) / F32(180))
    return Light(LIGHT_DIRECTIONAL, tuple(np.broadcast_to(radiance, 3)),
                 tuple(direction), rad)


def EnvLight(texel, scaler: float = 1.0, rot: float = 0.0) -> Light:
    """CreateEnvLight with a constant texture (core/light/env_light.cpp)."""
    return Light(LIGHT_ENV, tuple(np.broadcast_to(texel, 3)), scaler=scaler,
                 rot=rot)


# -------------------------------------------------------------- primitives --
@dataclass
class Quad:
    """CreateQuad with identity transform (core/geometry/quad.cpp:36-50)."""
    a: Sequence[float]
    b: Sequence[float]
    c: Sequence[float]
    d: Sequence[float]
    material: int = 0
    two_sided: bool = False
    kind: int = 0
    emission: Optional[Sequence[float]] = None  # radiance: an area light


@dataclass
class Cube:
    """CreateCube (core/geometry/cube.cpp:35-76); ``transform`` holds the 16
    row-major entries a YAML ``transform`` carries."""
    transform: Sequence[float]
    material: int = 0
    two_sided: bool = False
    kind: int = 1
    emission: Optional[Sequence[float]] = None


@dataclass
class Mesh:
    """Triangle mesh (MeshGeo, core/geometry/mesh.cpp:52-306)."""
    positions: np.ndarray
    indices: np.ndarray
    normals: Optional[np.ndarray] = None
    material: int = 0
    two_sided: bool = False
    kind: int = 2
    emission: Optional[Sequence[float]] = None


@dataclass
class Camera:
    """Thin-lens camera arguments (factory/creator/camera_creators.cpp)."""
    position: Sequence[float]
    look_at: Sequence[float]
    up: Sequence[float]
    fov: float              # degrees
    width: int
    height: int
    lens_radius: float = 0.0
    focal_distance: float = 1.0
    matrices: Optional[np.ndarray] = None  # [36] override (exact reference)

    def pack(self) -> np.ndarray:
        if self.matrices is not None:
            return np.asarray(self.matrices, F32)
        return camera_matrices(self)

    def harness_pack(self) -> np.ndarray:
        return np.array([*self.position, *self.look_at, *self.up, self.fov,
                         self.lens_radius, self.focal_distance], F32)


@dataclass
class Scene:
    primitives: List = field(default_factory=list)
    materials: List[Material] = field(default_factory=list)
    lights: List[Light] = field(default_factory=list)
    camera: Optional[Camera] = None


# -------------------------------------------------------------- flattening --
# Corner table of the unit cube, face by face (core/geometry/cube.cpp:36-61).
_CUBE_VERTS = np.array([
    [[-.5, -.5, -.5], [-.5, -.5, .5], [.5, -.5, .5], [.5, -.5, -.5]],
    [[-.5, .5, .5], [-.5, .5, -.5], [.5, .5, -.5], [.5, .5, .5]],
    [[-.5, .5, -.5], [-.5, -.5, -.5], [.5, -.5, -.5], [.5, .5, -.5]],
    [[.5, .5, .5], [.5, -.5, .5], [-.5, -.5, .5], [-.5, .5, .5]],
    [[-.5, .5, .5], [-.5, -.5, .5], [-.5, -.5, -.5], [-.5, .5, -.5]],
    [[.5, .5, -.5], [.5, -.5, -.5], [.5, -.5, .5], [.5, .5, .5]],
], F32)


def yaml_matrix(rowmajor16) -> np.ndarray:
    """Column-major 4x4 from 16 row-major entries, reading the first 15 as
    the YAML decoder does (factory/creator/helper.h:83-92)."""
    m = np.eye(4, dtype=F32)  # m[col][row]
    v = np.asarray(rowmajor16, F32)
    for i in range(15):
        m[i % 4][i // 4] = v[i]
    return m


def transform_point(m_colmajor: np.ndarray, p: np.ndarray) -> np.ndarray:
    """Matrix4::transformPoint (math/matrix4.h:115-118) in float32, summing
    the columns in order and dividing by w, for points p [n,3]."""
    p = np.asarray(p, F32)
    out = np.zeros((p.shape[0], 4), F32)
    hom = np.concatenate([p, np.ones((p.shape[0], 1), F32)], axis=1)
    for row in range(4):
        acc = np.zeros(p.shape[0], F32)
        for pos in range(4):
            acc = acc + m_colmajor[pos][row] * hom[:, pos]
        out[:, row] = acc
    return out[:, :3] / out[:, 3:4]


def _prim_triangles(p):
    """(tris [n,3,3], corner normals [n,3,3] or None, flags) of a primitive
    in the reference's MeshView order."""
    if p.kind == 0:
        a, b, c, d = (np.asarray(x, F32) for x in (p.a, p.b, p.c, p.d))
        tris = np.stack([np.stack([a, b, c]), np.stack([a, c, d])])
        flags = 0
        cn = None
    elif p.kind == 1:
        m = yaml_matrix(p.transform)
        pos = transform_point(m, _CUBE_VERTS.reshape(-1, 3))
        tris = []
        for i in range(6):
            idx = 4 * i
            # tuples (idx, idx+2, idx+1) and (idx, idx+3, idx+2); libstdc++
            # stores a tuple's members in reverse, so the MeshView sees k,j,i
            for (ti, tj, tk) in ((idx, idx + 2, idx + 1), (idx, idx + 3, idx + 2)):
                tris.append(np.stack([pos[tk], pos[tj], pos[ti]]))
        tris = np.stack(tris)
        flags = TRI_NG_REVERSED
        cn = None
    else:
        pos = np.asarray(p.positions, F32)
        idx = np.asarray(p.indices, np.int64).reshape(-1, 3)
        tris = pos[idx]
        flags = 0
        cn = None
        if p.normals is not None:
            flags |= TRI_HAS_NORMALS
            cn = np.asarray(p.normals, F32)[idx]
    if p.two_sided:
        flags |= TRI_TWO_SIDED
    return tris.astype(F32), cn, flags


def _prim_bounds(p, tris):
    if p.kind == 2:
        pos = np.asarray(p.positions, F32)
        return pos.min(0), pos.max(0)
    v = tris.reshape(-1, 3)
    return v.min(0), v.max(0)


def _join(a, b):
    """Bounds::Join (math/bounds.h:108-113): a point box is absorbed."""
    if np.array_equal(a[0], a[1]):
        return b
    if np.array_equal(b[0], b[1]):
        return a
    return np.minimum(a[0], b[0]), np.maximum(a[1], b[1])


@dataclass
class FlatScene:
    tris: np.ndarray        # [n, 9] float32
    corner_n: np.ndarray    # [n, 9] float32
    tri_mat: np.ndarray     # [n] int32
    tri_flags: np.ndarray   # [n] int32
    world: np.ndarray       # [6] float32
    materials: np.ndarray   # [m, 16] float32
    lights: np.ndarray      # [l, 12] float32
    camera: Optional[np.ndarray]  # [36] float32
    # emissive primitives (area lights), in primitive order: radiance, and
    # first triangle, triangle count, geometry kind (0 quad, 1 cube, 2 mesh),
    # two_sided
    emit_rad: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), F32))
    emit_info: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))

    @property
    def n_tris(self) -> int:
        return int(self.tris.shape[0])


def flatten(scene: Scene) -> FlatScene:
    tris, cns, mats, flags = [], [], [], []
    emit_rad, emit_info = [], []
    n = 0
    world = (np.full(3, np.finfo(F32).max, F32),
             np.full(3, -np.finfo(F32).max, F32))
    for p in scene.primitives:
        t, cn, fl = _prim_triangles(p)
        e = getattr(p, "emission", None)
        if e is not None and np.any(np.asarray(e, F32) != 0):
            emit_rad.append(np.broadcast_to(np.asarray(e, F32), 3))
            emit_info.append([n, t.shape[0], p.kind, int(p.two_sided)])
        n += t.shape[0]
        tris.append(t.reshape(-1, 9))
        cns.append(np.zeros((t.shape[0], 9), F32) if cn is None
                   else cn.reshape(-1, 9).astype(F32))
        mats.append(np.full(t.shape[0], p.material, np.int32))
        flags.append(np.full(t.shape[0], fl, np.int32))
        world = _join(world, _prim_bounds(p, t))
    mat_arr = (np.stack([m.pack() for m in scene.materials])
               if scene.materials else np.zeros((0, 16), F32))
    light_arr = (np.stack([l.pack() for l in scene.lights])
                 if scene.lights else np.zeros((0, 12), F32))
    return FlatScene(
        tris=np.ascontiguousarray(np.concatenate(tris), F32),
        corner_n=np.ascontiguousarray(np.concatenate(cns), F32),
        tri_mat=np.concatenate(mats),
        tri_flags=np.concatenate(flags),
        world=np.concatenate(world).astype(F32),
        materials=mat_arr.astype(F32),
        lights=light_arr.astype(F32),
        camera=None if scene.camera is None else scene.camera.pack(),
        emit_rad=np.array(emit_rad, F32).reshape(-1, 3),
        emit_info=np.array(emit_info, np.int32).reshape(-1, 4))


# ----------------------------------------------------------------- camera --
def camera_matrices(cam: Camera) -> np.ndarray:
    """raster2camera and camera2world of ThinLensCamera
    (core/camera/thin_lens.cpp:40-54), computed in float64 and rounded once.
    Returns the [36] camera record: two column-major 4x4 matrices, lens
    radius, focal distance, width, height."""
    eye = np.asarray(cam.position, np.float64)
    tgt = np.asarray(cam.look_at, np.float64)
    up = np.asarray(cam.up, np.float64)
    back = eye - tgt
    back /= np.linalg.norm(back)
    right = np.cross(up, back)
    right /= np.linalg.norm(right)
    rup = np.cross(back, right)
    rup /= np.linalg.norm(rup)
    c2w = np.eye(4)
    c2w[:3, 0], c2w[:3, 1], c2w[:3, 2], c2w[:3, 3] = right, rup, back, eye
    W, H = float(cam.width), float(cam.height)
    near, far = 1.0, 1000.0
    fov = float(F32(cam.fov) * F32(3.141592654) / F32(180))
    aspect = W / H
    # math/matrix4.h:61-66: size = 2 near tan(fov/2) * (aspect, 1)
    size = 2.0 * near * math.tan(fov * 0.5) * np.array([aspect, 1.0])
    # math/matrix4.h:139-157: the y scale is negated (yScale(-1))
    xs = 2 * near / size[0]
    ys = 2 * near / size[1] * -1.0
    zs = 1.0 / (far - near)
    proj = np.array([[xs, 0, 0, 0], [0, ys, 0, 0],
                     [0, 0, near * zs, near * zs * far], [0, 0, -1, 0]])
    s2r = (np.diag([W, H, 1.0, 1.0]) @ np.diag([0.5, -0.5, 1.0, 1.0]) @
           np.array([[1, 0, 0, 1.0], [0, 1, 0, -1.0], [0, 0, 1, 0],
                     [0, 0, 0, 1]]))
    r2c = np.linalg.inv(proj) @ np.linalg.inv(s2r)
    out = np.zeros(36, F32)
    out[0:16] = r2c.T.reshape(-1)   # column-major
    out[16:32] = c2w.T.reshape(-1)
    out[32], out[33] = cam.lens_radius, cam.focal_distance
    out[34], out[35] = cam.width, cam.height
    return out


# ------------------------------------------------------- synthetic scenes --
def _rot_y_matrix_rowmajor(scale, angle_deg, translate):
    """Row-major 16 entries of translate * R_y(angle) * scale."""
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    sx, sy, sz = scale
    tx, ty, tz = translate
    m = np.array([[c * sx, 0, s * sz, tx],
                  [0, sy, 0, ty],
                  [-s * sx, 0, c * sz, tz],
                  [0, 0, 0, 1]], np.float64)
    return m.astype(F32).reshape(-1)


def cornell_box(width: int = 256, height: int = 256) -> Scene:
    """The plain PT-MIS Cornell-style box: a 1-unit box of 5 walls (open
    front, 10 triangles), two inner boxes (24 triangles) rotated +15 and -18
    degrees about y, Lambertian albedos white 0.73, red (0.65,0.05,0.05),
    green (0.12,0.45,0.15), a directional light of radiance 3 travelling along
    (-0.3,-1,-0.2) (the reference's YAML key takes the direction toward the
    light, (0.3,1,0.2)), a constant environment of 0.2, and a pinhole camera
    with a 40 degree field of view."""
    white, red, green = 0, 1, 2
    mats = [Diffuse((0.73, 0.73, 0.73)), Diffuse((0.65, 0.05, 0.05)),
            Diffuse((0.12, 0.45, 0.15))]
    h = 0.5
    prims = [
        Quad((-h, -h, h), (h, -h, h), (h, -h, -h), (-h, -h, -h), white, True),   # floor
        Quad((-h, h, -h), (h, h, -h), (h, h, h), (-h, h, h), white, True),       # ceiling
        Quad((-h, -h, -h), (h, -h, -h), (h, h, -h), (-h, h, -h), white, True),   # back
        Quad((-h, -h, h), (-h, -h, -h), (-h, h, -h), (-h, h, h), red, True),     # left
        Quad((h, -h, -h), (h, -h, h), (h, h, h), (h, h, -h), green, True),       # right
        Cube(_rot_y_matrix_rowmajor((0.3, 0.6, 0.3), 15.0, (-0.17, -0.2, -0.12)), white, False),
        Cube(_rot_y_matrix_rowmajor((0.3, 0.3, 0.3), -18.0, (0.17, -0.35, 0.12)), white, False),
    ]
    lights = [DirectionalLight((0.3, 1.0, 0.2), 3.0), EnvLight(0.2)]
    cam = Camera((0.0, 0.0, 1.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0,
                 width, height)
    return Scene(prims, mats, lights, cam)


def cornell_area(width: int = 256, height: int = 256) -> Scene:
    """The box of ``cornell_box`` lit by its emitters, one of each kind the
    reference's area lights take: a one-sided ceiling quad facing down
    (radiance (8,6,3)), a two-sided vertical quad near the left wall
    (1,2,4), an emissive icosphere mesh of 80 triangles on the floor
    (6,2,1) and an emissive cube under the ceiling (2,4,2); beside them a
    directional light of radiance 1 and a constant environment of 0.05.
    The tall inner box is a Disney material, the short one Lambertian."""
    white, red, green, disney = 0, 1, 2, 3
    mats = [Diffuse((0.73, 0.73, 0.73)), Diffuse((0.65, 0.05, 0.05)),
            Diffuse((0.12, 0.45, 0.15)),
            Disney((0.8, 0.6, 0.4), metallic=0.3, roughness=0.35,
                   clearcoat=0.5, clearcoat_gloss=0.7)]
    h = 0.5
    v, f = icosphere(1)
    ball = (v * 0.07 + np.array([0.3, -h + 0.07, 0.28])).astype(F32)
    prims = [
        Quad((-h, -h, h), (h, -h, h), (h, -h, -h), (-h, -h, -h), white, True),   # floor
        Quad((-h, h, -h), (h, h, -h), (h, h, h), (-h, h, h), white, True),       # ceiling
        Quad((-h, -h, -h), (h, -h, -h), (h, h, -h), (-h, h, -h), white, True),   # back
        Quad((-h, -h, h), (-h, -h, -h), (-h, h, -h), (-h, h, h), red, True),     # left
        Quad((h, -h, -h), (h, -h, h), (h, h, h), (h, h, -h), green, True),       # right
        Cube(_rot_y_matrix_rowmajor((0.3, 0.6, 0.3), 15.0, (-0.17, -0.2, -0.12)), disney, False),
        Cube(_rot_y_matrix_rowmajor((0.3, 0.3, 0.3), -18.0, (0.17, -0.35, 0.12)), white, False),
        # emitters
        Quad((-0.15, h - 1e-3, -0.15), (0.15, h - 1e-3, -0.15),
             (0.15, h - 1e-3, 0.15), (-0.15, h - 1e-3, 0.15), white, False,
             emission=(8.0, 6.0, 3.0)),
        Quad((-0.42, -0.1, -0.25), (-0.42, -0.1, 0.0), (-0.42, 0.12, 0.0),
             (-0.42, 0.12, -0.25), white, True, emission=(1.0, 2.0, 4.0)),
        Mesh(ball, f.astype(np.int32), None, white, False,
             emission=(6.0, 2.0, 1.0)),
        Cube(_rot_y_matrix_rowmajor((0.08, 0.08, 0.08), 30.0, (0.25, 0.33, -0.3)),
             white, False, emission=(2.0, 4.0, 2.0)),
    ]
    lights = [DirectionalLight((0.3, 1.0, 0.2), 1.0), EnvLight(0.05)]
    cam = Camera((0.0, 0.0, 1.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0,
                 width, height)
    return Scene(prims, mats, lights, cam)


def material_box(width: int = 256, height: int = 256) -> Scene:
    """The box of ``cornell_box`` with the other materials: a plastic floor
    (ior 1.5, thickness 1, sigma_a 0.3), a mirror tall box, a rough gold-like
    metal short box, a glass ball of 320 smooth-shaded triangles (ior 1.5)
    on it, and a ceiling light quad of radiance (6,6,6) with the null
    material (rays pass through it); a directional light of radiance 1 and
    a constant environment of 0.1."""
    white, red, green, plastic, mirror, metal, glass, null = range(8)
    mats = [Diffuse((0.73, 0.73, 0.73)), Diffuse((0.65, 0.05, 0.05)),
            Diffuse((0.12, 0.45, 0.15)),
            Plastic((0.6, 0.55, 0.5), 1.5, 1.0, 0.3),
            Mirror((0.9, 0.9, 0.9)),
            Metal((1.0, 0.95, 0.9), (3.98, 2.38, 1.60), (0.14, 0.37, 1.44), 0.25, 0.15),
            Glass(1.5, (1.0, 1.0, 1.0), (0.9, 0.95, 1.0)),
            Null()]
    h = 0.5
    v, f = icosphere(2)
    ball = (v * 0.12 + np.array([0.17, -0.2 + 0.12, 0.12])).astype(F32)
    prims = [
        Quad((-h, -h, h), (h, -h, h), (h, -h, -h), (-h, -h, -h), plastic, True),  # floor
        Quad((-h, h, -h), (h, h, -h), (h, h, h), (-h, h, h), white, True),        # ceiling
        Quad((-h, -h, -h), (h, -h, -h), (h, h, -h), (-h, h, -h), white, True),    # back
        Quad((-h, -h, h), (-h, -h, -h), (-h, h, -h), (-h, h, h), red, True),      # left
        Quad((h, -h, -h), (h, -h, h), (h, h, h), (h, h, -h), green, True),        # right
        Cube(_rot_y_matrix_rowmajor((0.3, 0.6, 0.3), 15.0, (-0.17, -0.2, -0.12)), mirror, False),
        Cube(_rot_y_matrix_rowmajor((0.3, 0.3, 0.3), -18.0, (0.17, -0.35, 0.12)), metal, False),
        Mesh(ball, f.astype(np.int32), v.astype(F32), glass, False),
        Quad((-0.12, h - 1e-3, -0.12), (0.12, h - 1e-3, -0.12),
             (0.12, h - 1e-3, 0.12), (-0.12, h - 1e-3, 0.12), null, False,
             emission=(6.0, 6.0, 6.0)),
    ]
    lights = [DirectionalLight((0.3, 1.0, 0.2), 1.0), EnvLight(0.1)]
    cam = Camera((0.0, 0.0, 1.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0,
                 width, height)
    return Scene(prims, mats, lights, cam)


def icosphere(subdiv: int):
    """Unit icosphere: 20 * 4**subdiv triangles (vertices [v,3] float64,
    triangles [t,3] int64)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
                 np.int64)
    for _ in range(subdiv):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        nf = f.shape[0]
        m01, m12, m20 = (nv + inv[:nf], nv + inv[nf:2 * nf], nv + inv[2 * nf:])
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def _lattice(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) ^
         iy.astype(np.uint64) * np.uint64(0xD8163841) ^
         iz.astype(np.uint64) * np.uint64(0xCB1AB31F) ^
         np.uint64(seed * 0x9E3779B1 & 0xFFFFFFFF))
    h = (h ^ (h >> np.uint64(15))) * np.uint64(0x2C1B3C6D)
    h = (h ^ (h >> np.uint64(12))) * np.uint64(0x297A2D39)
    h = h ^ (h >> np.uint64(15))
    return (h & np.uint64(0xFFFFFF)).astype(np.float64) / float(0xFFFFFF) * 2 - 1


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3D value noise in [-1, 1] with smoothstep interpolation."""
    q = np.floor(p)
    f = p - q
    w = f * f * (3 - 2 * f)
    i = q.astype(np.int64) + (1 << 20)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                c = _lattice(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out += c * wx * wy * wz
    return out


def fbm(p: np.ndarray, seed: int, octaves: int = 4, lacunarity: float = 2.0,
        gain: float = 0.5, base_freq: float = 2.0) -> np.ndarray:
    amp, freq, out, norm = 1.0, base_freq, np.zeros(p.shape[0]), 0.0
    for o in range(octaves):
        out += amp * value_noise(p * freq, seed + 101 * o)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return out / norm


def displaced_icosphere(subdiv: int, seed: int, amplitude: float = 0.15,
                        radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Icosphere radially displaced by 4-octave fBm (amplitude relative to the
    radius); returns float32 positions, smooth vertex normals and int32
    triangle indices."""
    v, f = icosphere(subdiv)
    r = radius * (1.0 + amplitude * fbm(v, seed))
    pos = v * r[:, None] + np.asarray(center, np.float64)
    e0 = pos[f[:, 1]] - pos[f[:, 0]]
    e1 = pos[f[:, 2]] - pos[f[:, 0]]
    fn = np.cross(e0, e1)
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    return pos.astype(F32), vn.astype(F32), f.astype(np.int32)


def disney_params(rng: np.random.Generator) -> Material:
    """Disney parameters drawn per seed: baseColor U[0,1]^3, metallic U[0,1],
    roughness U[0.05,1], specular 0.5, clearcoat U[0,1], clearcoat_gloss
    U[0,1], sheen 0 and the remaining parameters 0."""
    return Disney(base_color=tuple(rng.uniform(0, 1, 3)),
                  metallic=float(rng.uniform(0, 1)),
                  roughness=float(rng.uniform(0.05, 1)), specular=0.5,
                  clearcoat=float(rng.uniform(0, 1)),
                  clearcoat_gloss=float(rng.uniform(0, 1)))


def icosphere_scene(subdiv: int = 8, seed: int = 0, width: int = 1024,
                    height: int = 1024, ground: bool = True) -> Scene:
    """The single-job workload: an icosphere of 20*4**subdiv triangles
    (subdivision 8: 1,310,720) displaced by 4-octave fBm of amplitude 0.15,
    with seeded Disney parameters, on a 2-triangle Lambertian ground plane,
    lit by a constant environment of 0.5 and a directional light of 2.0."""
    rng = np.random.default_rng(seed)
    pos, nrm, idx = displaced_icosphere(subdiv, seed)
    mats = [disney_params(rng), Diffuse((0.5, 0.5, 0.5))]
    prims = [Mesh(pos, idx, nrm, 0, False)]
    if ground:
        g, y = 8.0, -1.2
        prims.append(Quad((-g, y, g), (g, y, g), (g, y, -g), (-g, y, -g), 1, True))
    lights = [DirectionalLight((0.3, 1.0, 0.2), 2.0), EnvLight(0.5)]
    cam = Camera((0.0, 0.6, 3.6), (0.0, -0.1, 0.0), (0.0, 1.0, 0.0), 40.0,
                 width, height)
    return Scene(prims, mats, lights, cam)


# ------------------------------------------------------- mixed workloads --
def _orbit_camera(rng: np.random.Generator, width: int, height: int,
                  target=(0.0, -0.1, 0.0), dist: float = 3.6) -> Camera:
    """Pinhole camera on a seeded sphere around the scene, looking at its
    centre (azimuth U[0, 360), elevation U[5, 45] degrees)."""
    az = np.radians(rng.uniform(0.0, 360.0))
    el = np.radians(rng.uniform(5.0, 45.0))
    t = np.asarray(target, np.float64)
    pos = t + dist * np.array([np.cos(el) * np.sin(az), np.sin(el),
                               np.cos(el) * np.cos(az)])
    return Camera(tuple(pos), tuple(t), (0.0, 1.0, 0.0), 40.0, width, height)


def clutter_meshes(n_cubes: int, rng: np.random.Generator, groups: int,
                   extent: float = 1.0):
    """Random-box clutter: n_cubes boxes (12 triangles each) with random
    centres in [-extent, extent]^3, sizes and rotations about y, split into
    `groups` meshes (one material each).  Returns [(positions, indices)]."""
    c = rng.uniform(-extent, extent, (n_cubes, 3))
    size = rng.uniform(0.02, 0.25, (n_cubes, 3)) * extent
    ang = rng.uniform(0.0, 2 * np.pi, n_cubes)
    corners = np.array([[x, y, z] for x in (-.5, .5) for y in (-.5, .5)
                        for z in (-.5, .5)])                       # [8, 3]
    # outward-facing triangles of the 8-corner box
    faces = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5],
                      [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
                      [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], np.int64)
    local = corners[None] * size[:, None, :]                        # [n, 8, 3]
    ca, sa = np.cos(ang)[:, None], np.sin(ang)[:, None]
    x = local[..., 0] * ca + local[..., 2] * sa
    z = -local[..., 0] * sa + local[..., 2] * ca
    pos = np.stack([x, local[..., 1], z], -1) + c[:, None, :]      # [n, 8, 3]
    out = []
    for g in range(groups):
        sel = np.arange(g, n_cubes, groups)
        if not len(sel):
            continue
        p = pos[sel].reshape(-1, 3).astype(F32)
        idx = (faces[None] + 8 * np.arange(len(sel))[:, None, None]).reshape(-1, 3)
        out.append((p, idx.astype(np.int32)))
    return out


def mixed_scene(seed: int, target_tris: int, width: int, height: int) -> Scene:
    """A scene of the batched/served workload: either a displaced icosphere
    at the smallest subdivision with at least `target_tris` triangles (at
    most subdivision 8), or random-box clutter of target_tris / 12 boxes in 16
    material groups; Disney parameters drawn per object, a 2-triangle
    Lambertian ground, a constant environment of 0.5 and a directional light
    of 2.0, and a camera on a seeded sphere around the scene."""
    rng = np.random.default_rng(seed)
    prims, mats = [], []
    if rng.uniform() < 0.5:
        s = 0
        while 20 * 4 ** s < target_tris and s < 8:
            s += 1
        pos, nrm, idx = displaced_icosphere(s, seed)
        mats.append(disney_params(rng))
        prims.append(Mesh(pos, idx, nrm, 0, False))
    else:
        for k, (p, idx) in enumerate(clutter_meshes(max(1, target_tris // 12), rng, 16)):
            mats.append(disney_params(rng))
            prims.append(Mesh(p, idx, None, k, False))
    mats.append(Diffuse((0.5, 0.5, 0.5)))
    g, y = 8.0, -1.2
    prims.append(Quad((-g, y, g), (g, y, g), (g, y, -g), (-g, y, -g), len(mats) - 1, True))
    lights = [DirectionalLight((0.3, 1.0, 0.2), 2.0), EnvLight(0.5)]
    return Scene(prims, mats, lights, _orbit_camera(rng, width, height))


def batch_workload(n: int = 48, seed: int = 0, resolutions=(128, 256, 512, 1024),
                   spp_range=(16, 256), tri_range=(1_000, 2_000_000)):
    """Job list of the batched workload: per job a scene seed, a triangle
    count log-uniform in tri_range, a square resolution drawn from
    `resolutions` and spp log-uniform in spp_range."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n):
        tris = int(round(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1])))))
        res = int(rng.choice(resolutions))
        spp = int(round(np.exp(rng.uniform(np.log(spp_range[0]), np.log(spp_range[1])))))
        jobs.append({"scene_seed": int(seed * 1000 + i), "tris": tris, "res": res,
                     "spp": spp})
    return jobs


def _rotation(rng: np.random.Generator) -> np.ndarray:
    """A uniformly random 3x3 rotation (QR of a Gaussian matrix)."""
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q *= np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def project(camera: Camera, points: np.ndarray) -> np.ndarray:
    """Raster coordinates (x, y) of world points through the camera's
    matrices (the inverse of the ray generation's mapping)."""
    m = np.asarray(camera.pack(), np.float64)
    r2c = m[0:16].reshape(4, 4).T
    c2w = m[16:32].reshape(4, 4).T
    w2r = np.linalg.inv(r2c) @ np.linalg.inv(c2w)
    p = np.concatenate([points, np.ones((len(points), 1))], 1) @ w2r.T
    return p[:, :2] / p[:, 3:4]


def large_scene(seed: int = 0, width: int = 1920, height: int = 1080,
                copies: int = 20, subdiv: int = 8, box: float = 100.0) -> Scene:
    """The precision-stress workload: `copies` copies of the single-job
    displaced icosphere (subdivision 8: 26,214,400 triangles for 20), each
    with a random rotation, a uniform scale U[0.5, 2] and a position inside
    a box^3 cube, flattened into one tree, each with its own Disney
    parameters; a constant environment of 0.5 and a directional light of
    2.0; a pinhole camera outside the cube looking at its centre."""
    rng = np.random.default_rng(seed)
    pos0, nrm0, idx = displaced_icosphere(subdiv, seed)
    pos0 = pos0.astype(np.float64)
    nrm0 = nrm0.astype(np.float64)
    prims, mats, centers, scales = [], [], [], []
    half = box / 2.0
    for k in range(copies):
        rot = _rotation(rng)
        scale = rng.uniform(0.5, 2.0)
        t = rng.uniform(-half + 2.5 * scale, half - 2.5 * scale, 3)
        pos = (pos0 @ rot.T) * scale + t
        nrm = nrm0 @ rot.T
        mats.append(disney_params(rng))
        prims.append(Mesh(pos.astype(F32), idx, nrm.astype(F32), k, False))
        centers.append(t)
        scales.append(scale)
    lights = [DirectionalLight((0.3, 1.0, 0.2), 2.0), EnvLight(0.5)]
    cam = Camera((0.0, 0.35 * box, 1.55 * box), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0,
                 width, height)
    scene = Scene(prims, mats, lights, cam)
    scene.copy_centers = np.array(centers)
    scene.copy_scales = np.array(scales)
    return scene
