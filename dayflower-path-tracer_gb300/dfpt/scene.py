"""Compiled scenes: the reference's 14 arrays + camera, the scene builder and the .scene file.

CompiledScene mirrors org.dayflower.pathtracer.scene.compiler.CompiledScene
(src/main/java/org/dayflower/pathtracer/scene/compiler/CompiledScene.java:55-71); its read/write
follow CompiledScene.read/write (CompiledScene.java:273-291, 353-373): a Java DataOutputStream
UTF name, then each array as a big-endian int length followed by big-endian elements
(util/Arrays2.java:56-66, 247-273).
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, f32p, i32p, ptr

# Material, shape and texture type ids (scene/material/*.java, scene/shape/*.java, scene/texture/*.java).
CLEAR_COAT, GLASS, LAMBERTIAN, PHONG, REFLECTION = 1, 2, 3, 4, 5
PLANE, SPHERE, TERRAIN, TRIANGLE, TRIANGLE_MESH = 1, 2, 3, 4, 5
TEX_BLEND, TEX_BULLSEYE, TEX_CHECKERBOARD, TEX_CONSTANT, TEX_FBM, TEX_IMAGE, TEX_SURFACE_NORMAL, TEX_UV = range(1, 9)

FLOAT_ARRAYS = ("point2fs", "point3fs", "vector3fs", "spheres", "terrains", "textures", "surfaces",
                "primitives_object_to_world", "primitives_world_to_object", "camera")
INT_ARRAYS = ("planes", "triangles", "bounding_volume_hierarchies", "primitives")
# The order CompiledScene.write uses.
FILE_ORDER = (("point2fs", "f"), ("point3fs", "f"), ("vector3fs", "f"), ("planes", "i"), ("spheres", "f"),
              ("terrains", "f"), ("triangles", "i"), ("bounding_volume_hierarchies", "i"), ("textures", "f"),
              ("surfaces", "f"), ("primitives", "i"), ("primitives_object_to_world", "f"),
              ("primitives_world_to_object", "f"), ("camera", "f"))


def pack_argb(r: float, g: float, b: float, a: float = 1.0) -> float:
    """Color.pack() (image4j Color.java:1493-1514): ARGB8 of clamped components, stored as float."""
    def q(x):
        x = min(max(float(np.float32(x)), 0.0), 1.0)
        return int(np.float32(np.float32(x) * np.float32(255.0) + np.float32(0.5)))
    v = ((q(a) & 0xFF) << 24) | ((q(r) & 0xFF) << 16) | ((q(g) & 0xFF) << 8) | (q(b) & 0xFF)
    if v >= 1 << 31:
        v -= 1 << 32
    return float(np.float32(v))


@dataclass
class CompiledScene:
    name: str = "scene"
    point2fs: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    point3fs: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    vector3fs: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    planes: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int32))
    spheres: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    terrains: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    triangles: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int32))
    bounding_volume_hierarchies: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int32))
    textures: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    surfaces: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    primitives: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    primitives_object_to_world: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    primitives_world_to_object: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    camera: np.ndarray = field(default_factory=lambda: np.zeros(19, np.float32))
    # Optional per-primitive extension records {Phong exponent, emission scale r, g, b} (empty: none;
    # see dfpt_scene_desc.primitive_extensions). Not part of the reference's arrays or .scene file.
    primitive_extensions: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))

    def __post_init__(self):
        for k in FLOAT_ARRAYS:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float32))
        for k in INT_ARRAYS:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))
        self.primitive_extensions = np.ascontiguousarray(self.primitive_extensions, dtype=np.float32).reshape(-1)

    @property
    def primitive_count(self) -> int:
        return len(self.primitives) // 3

    def desc(self) -> _lib.SceneDesc:
        """A dfpt_scene_desc pointing at these arrays (keep the scene alive while it is used)."""
        d = _lib.SceneDesc()
        for k in FLOAT_ARRAYS + INT_ARRAYS:
            a = getattr(self, k)
            setattr(d, k if k != "bounding_volume_hierarchies" else "bounding_volume_hierarchies",
                    ptr(a, C.c_float if k in FLOAT_ARRAYS else C.c_int32))
            setattr(d, k + "_count", int(a.size))
        if self.primitive_extensions.size:
            d.primitive_extensions = ptr(self.primitive_extensions, C.c_float)
            d.primitive_extensions_count = int(self.primitive_extensions.size)
        return d

    def arrays(self) -> dict:
        return {k: getattr(self, k) for k in FLOAT_ARRAYS + INT_ARRAYS}

    def copy(self) -> "CompiledScene":
        return CompiledScene(self.name, **{k: v.copy() for k, v in self.arrays().items()},
                             primitive_extensions=self.primitive_extensions.copy())

    def save_npz(self, path) -> None:
        np.savez_compressed(path, name=np.array(self.name), primitive_extensions=self.primitive_extensions, **self.arrays())

    @staticmethod
    def load_npz(path) -> "CompiledScene":
        z = np.load(path, allow_pickle=False)
        ext = z["primitive_extensions"] if "primitive_extensions" in z.files else np.zeros(0, np.float32)
        return CompiledScene(str(z["name"]), **{k: z[k] for k in FLOAT_ARRAYS + INT_ARRAYS}, primitive_extensions=ext)

    # -- the reference's .scene file ---------------------------------------------------------
    def write(self, path) -> None:
        name = self.name.encode("utf-8")
        with open(path, "wb") as f:
            f.write(struct.pack(">H", len(name)) + name)
            for key, kind in FILE_ORDER:
                a = getattr(self, key)
                f.write(struct.pack(">i", int(a.size)))
                f.write(a.astype(">f4" if kind == "f" else ">i4").tobytes())

    @staticmethod
    def read(path) -> "CompiledScene":
        with open(path, "rb") as f:
            data = f.read()
        (n,) = struct.unpack_from(">H", data, 0)
        pos = 2
        name = data[pos:pos + n].decode("utf-8")
        pos += n
        arrays = {}
        for key, kind in FILE_ORDER:
            if pos + 4 > len(data):
                raise ValueError(f"truncated .scene file at {key}")
            (length,) = struct.unpack_from(">i", data, pos)
            pos += 4
            if length < 0 or pos + 4 * length > len(data):
                raise ValueError(f"bad length {length} for {key}")
            a = np.frombuffer(data, dtype=">f4" if kind == "f" else ">i4", count=length, offset=pos)
            arrays[key] = a.astype(np.float32 if kind == "f" else np.int32)
            pos += 4 * length
        return CompiledScene(name, **arrays)


def camera_set_resolution(camera: np.ndarray, width, height) -> np.ndarray:
    """Camera.setResolution (scene/Camera.java:806-816) on a 19-float camera record, in place: the
    resolution, then the vertical field of view from the horizontal one (setFieldOfViewX,
    Camera.java:743-748, with Math4J's float-rounded trigonometry). DayflowerApplication sets the
    camera to the kernel's size before rendering (DayflowerApplication.java:334)."""
    rx, ry = np.float32(width), np.float32(height)
    camera[16], camera[17] = rx, ry
    fov_x = np.float32(camera[4])
    rad = np.float32(np.float64(fov_x) * (np.pi / 180.0))
    tn = np.float32(np.tan(np.float64(np.float32(rad * np.float32(0.5)))))
    at = np.float32(np.arctan(np.float64(np.float32(tn * np.float32(ry / rx)))))
    camera[5] = np.float32(np.float64(np.float32(np.float32(2.0) * at)) * (180.0 / np.pi))
    return camera


class SkyState:
    """Sky.set(sunDirectionWorld, turbidity) (scene/Sky.java:295-333) as a dfpt_sky."""

    def __init__(self, sun_direction_world=(1.0, 1.0, 1.0), turbidity: float = 2.0):
        self.raw = _lib.Sky()
        self.set(sun_direction_world, turbidity)

    def set(self, sun_direction_world, turbidity: float) -> None:
        d = np.asarray(sun_direction_world, dtype=np.float32)
        check(_lib.load().dfpt_sky_set(C.byref(self.raw), ptr(d, C.c_float), float(turbidity)))
        self.sun_direction_world_input = tuple(float(x) for x in d)
        self.turbidity = float(turbidity)

    def as_dict(self) -> dict:
        r = self.raw
        return {
            "perez_relative_luminance": list(r.perez_relative_luminance), "perez_x": list(r.perez_x),
            "perez_y": list(r.perez_y), "zenith_relative_luminance": r.zenith_relative_luminance,
            "zenith_x": r.zenith_x, "zenith_y": r.zenith_y, "theta": r.theta,
            "orthonormal_basis_u": list(r.orthonormal_basis_u), "orthonormal_basis_v": list(r.orthonormal_basis_v),
            "orthonormal_basis_w": list(r.orthonormal_basis_w), "sun_direction": list(r.sun_direction),
            "sun_direction_world": list(r.sun_direction_world), "sun_origin": list(r.sun_origin),
            "is_sky_active": r.is_sky_active, "is_sun_active": r.is_sun_active,
        }

    @staticmethod
    def from_dict(d: dict) -> "SkyState":
        s = SkyState.__new__(SkyState)
        s.raw = _lib.Sky()
        for k, v in d.items():
            cur = getattr(s.raw, k)
            if hasattr(cur, "__len__"):
                for i, x in enumerate(v):
                    cur[i] = x
            else:
                setattr(s.raw, k, v)
        return s


class SceneBuilder:
    """Flat description of a Scene, compiled by the C++ restatement of SceneCompiler."""

    def __init__(self):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.dfpt_builder_create(C.byref(h)))
        self._h = h
        self._ext = []  # per primitive: (Phong exponent, emission scale r, g, b)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.dfpt_builder_destroy(h)
            self._h = None

    # Textures (Texture.toArray layouts).
    def texture(self, record) -> int:
        rec = np.asarray(record, dtype=np.float32)
        return check(self._lib.dfpt_builder_add_texture(self._h, ptr(rec, C.c_float), int(rec.size)))

    def constant(self, r, g, b) -> int:
        return self.texture([TEX_CONSTANT, 3, pack_argb(r, g, b)])

    def checkerboard(self, c0, c1, degrees=0.0, scale_u=1.0, scale_v=1.0) -> int:
        rad = np.float32(np.float64(np.float32(degrees)) * (np.pi / 180.0))  # MathF.toRadians
        return self.texture([TEX_CHECKERBOARD, 8, pack_argb(*c0), pack_argb(*c1), float(np.cos(np.float64(rad))),
                             float(np.sin(np.float64(rad))), scale_u, scale_v])

    def fbm(self, addend, multiplier, frequency, gain, octaves) -> int:
        return self.texture([TEX_FBM, 7, pack_argb(*addend), pack_argb(*multiplier), frequency, gain, octaves])

    def blend(self, texture_a, texture_b, factor=0.5) -> int:
        """BlendTexture (texture/BlendTexture.java:206-214): the children are earlier builder
        textures; the compiler writes their offsets into the record."""
        return self.texture([TEX_BLEND, 5, texture_a, texture_b, factor])

    def bullseye(self, color_a=(1.0, 0.0, 0.0), color_b=(0.0, 0.0, 0.0)) -> int:
        return self.texture([TEX_BULLSEYE, 4, pack_argb(*color_a), pack_argb(*color_b)])

    def surface_normal_texture(self, tangent_space=False) -> int:
        return self.texture([TEX_SURFACE_NORMAL, 3, 1.0 if tangent_space else 0.0])

    def uv_texture(self) -> int:
        return self.texture([TEX_UV, 2])

    def image(self, width, height, rgb, degrees=0.0, scale_u=1.0, scale_v=1.0) -> int:
        """ImageTexture (texture/ImageTexture.java:337-357): `rgb` holds width x height 0x00RRGGBB
        ints, top row first (see dfpt.images.load)."""
        data = np.asarray(rgb, dtype=np.int64).reshape(-1)
        if data.size != int(width) * int(height):
            raise ValueError("image data does not match width x height")
        rad = np.float32(np.float64(np.float32(degrees)) * (np.pi / 180.0))  # MathF.toRadians
        head = [TEX_IMAGE, 8 + data.size, float(np.cos(np.float64(rad))), float(np.sin(np.float64(rad))), width, height,
                scale_u, scale_v]
        rec = np.concatenate([np.asarray(head, np.float32), data.astype(np.float32)])
        return self.texture(rec)

    def image_file(self, path, degrees=0.0, scale_u=1.0, scale_v=1.0) -> int:
        """ImageTexture.load(file, degrees, scaleU, scaleV)."""
        from . import images

        w, h, rgb = images.load(path)
        return self.image(w, h, rgb, degrees, scale_u, scale_v)

    def surface(self, material, albedo, emission, normal, noise_amount=0.0, noise_scale=0.0) -> int:
        return check(self._lib.dfpt_builder_add_surface(self._h, material, albedo, emission, normal,
                                                       float(noise_amount), float(noise_scale)))

    # Shapes.
    def plane(self, a, b, c) -> int:
        p = np.asarray(list(a) + list(b) + list(c), dtype=np.float32)
        return check(self._lib.dfpt_builder_add_shape(self._h, PLANE, ptr(p, C.c_float)))

    def sphere(self, position, radius) -> int:
        p = np.asarray(list(position) + [radius], dtype=np.float32)
        return check(self._lib.dfpt_builder_add_shape(self._h, SPHERE, ptr(p, C.c_float)))

    def terrain(self, frequency, gain, minimum, maximum, octaves) -> int:
        p = np.asarray([frequency, gain, minimum, maximum, octaves], dtype=np.float32)
        return check(self._lib.dfpt_builder_add_shape(self._h, TERRAIN, ptr(p, C.c_float)))

    def mesh(self, positions, indices, normals=None, uvs=None, tangents=None, as_mesh=True) -> int:
        pos = np.asarray(positions, dtype=np.float32).reshape(-1, 3)
        nv = len(pos)
        v = np.zeros((nv, 11), dtype=np.float32)
        v[:, 0:3] = pos
        if normals is not None:
            v[:, 3:6] = np.asarray(normals, dtype=np.float32).reshape(-1, 3)
        if uvs is not None:
            v[:, 6:8] = np.asarray(uvs, dtype=np.float32).reshape(-1, 2)
        if tangents is not None:
            v[:, 8:11] = np.asarray(tangents, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int32).reshape(-1, 3))
        v = np.ascontiguousarray(v)
        return check(self._lib.dfpt_builder_add_mesh(self._h, ptr(v, C.c_float), nv, ptr(idx, C.c_int32), len(idx),
                                                    1 if as_mesh else 0))

    def primitive(self, shape, surface, position=(0, 0, 0), rotation=(0, 0, 0, 1), scale=(1, 1, 1),
                  phong_exponent=None, emission_scale=None) -> int:
        """A primitive (Primitive: shape, surface, Transform). `phong_exponent` (the exponent a
        PhongMaterial holds, which SceneCompiler drops) and `emission_scale` (a factor on the
        emission texture's 8-bit colour, for HDR emitters) go into the scene's extension records;
        without them the primitive renders as the reference's (exponent 50, scale 1)."""
        t = np.asarray(list(position) + list(rotation) + list(scale), dtype=np.float32)
        idx = check(self._lib.dfpt_builder_add_primitive(self._h, shape, surface, ptr(t, C.c_float)))
        es = (1.0, 1.0, 1.0) if emission_scale is None else tuple(float(v) for v in np.broadcast_to(emission_scale, (3,)))
        rec = (50.0 if phong_exponent is None else float(phong_exponent),) + es
        self._ext.append((rec, phong_exponent is not None or emission_scale is not None))
        return idx

    def camera(self, eye, look_at, field_of_view_x=90.0, resolution=(800, 800), aperture_radius=0.0,
               focal_distance=30.0, fisheye=False) -> None:
        e = np.asarray(eye, dtype=np.float32)
        la = np.asarray(look_at, dtype=np.float32)
        check(self._lib.dfpt_builder_set_camera(self._h, ptr(e, C.c_float), ptr(la, C.c_float), float(field_of_view_x),
                                               float(resolution[0]), float(resolution[1]), float(aperture_radius),
                                               float(focal_distance), 2 if fisheye else 1))

    def compile(self, name: str = "scene", threads: int = 0, exhaustive_bvh: bool = False) -> CompiledScene:
        """SceneCompiler.compile. `exhaustive_bvh` runs the builder's split search as the reference's
        loop over every item for every candidate (slow; the default sorted sweep gives the same tree)."""
        out = C.c_void_p()
        check(self._lib.dfpt_builder_set_exhaustive(self._h, 1 if exhaustive_bvh else 0))
        check(self._lib.dfpt_builder_compile(self._h, int(threads), C.byref(out)))
        try:
            d = _lib.SceneDesc()
            check(self._lib.dfpt_compiled_describe(out, C.byref(d)))
            arrays = {}
            for k in FLOAT_ARRAYS + INT_ARRAYS:
                n = getattr(d, k + "_count")
                p = getattr(d, k)
                dtype = np.float32 if k in FLOAT_ARRAYS else np.int32
                arrays[k] = np.ctypeslib.as_array(p, shape=(n,)).astype(dtype, copy=True) if n else np.zeros(0, dtype)
            # The compiler keeps the primitives in the order they were added.
            ext = np.asarray([r for r, _ in self._ext], np.float32).reshape(-1) if any(u for _, u in self._ext) \
                else np.zeros(0, np.float32)
            return CompiledScene(name, **arrays, primitive_extensions=ext)
        finally:
            self._lib.dfpt_compiled_destroy(out)
