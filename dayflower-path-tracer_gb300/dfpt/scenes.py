"""The reference's named scenes (src/main/java/org/dayflower/pathtracer/scene/loader/Scenes.java:
81-480), built with SceneBuilder from a resource directory that holds `model/` and `texture/`
(the layout of the reference's resources/distribution/resources; Scenes.java:482-492).

`scene_by_name(directory, name)` dispatches as Scenes.getSceneByName (Scenes.java:81-104; unknown
names give the material showcase) and returns (CompiledScene, SkyState). A scene whose model or
texture file is missing raises FileNotFoundError, as the reference's loaders throw. Each scene is
written as the reference builds it: the same primitives in the same order, the same shapes,
transforms, materials, textures (ImageTexture.load through dfpt.images) and camera eye; the camera
is the reference's default (Camera.java:239-254: eye (55, 42, 155.6), pitch 0, yaw 0, field of view
90 degrees, focal distance 30, 800 x 800, thin lens), the sky Sky() (sun direction (1, 1, 1),
turbidity 2).
"""
from __future__ import annotations

import os

import numpy as np

from . import obj as _obj
from .scene import (CLEAR_COAT, GLASS, LAMBERTIAN, PHONG, REFLECTION, CompiledScene, SceneBuilder, SkyState,
                    camera_set_resolution)

F = np.float32

# image4j Color constants (Color.java) and Color(int, int, int) = component / 255.0F.
BLACK = (0.0, 0.0, 0.0)
WHITE = (1.0, 1.0, 1.0)
GRAY = (0.5, 0.5, 0.5)
RED = (1.0, 0.0, 0.0)
GREEN = (0.0, 1.0, 0.0)
BLUE = (0.0, 0.0, 1.0)
ORANGE = (1.0, 0.5, 0.0)


def rgb255(r, g, b):
    return tuple(float(F(v) / F(255.0)) for v in (r, g, b))


GROUND = ((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), (1.0, 0.0, 0.0))  # Plane through (0,0,0), (0,0,1), (1,0,0)

NAMES = ("Girl_Scene", "House_Scene", "House_2_Scene", "Image_Scene", "Material_Showcase_Scene", "Monkey_Scene",
         "Terrain_Scene", "Wine_Glass_Scene", "Zealot_Scene")


def model_path(directory, name):
    return os.path.join(str(directory), "model", name)


def texture_path(directory, name):
    return os.path.join(str(directory), "texture", name)


def _require(path):
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    return path


def default_basis():
    """U, V, W of `new Camera()` (Camera.java:239-254, update at :877-946): pitch =
    AngleF.pitch(x axis) = 0 and yaw = AngleF.yaw(y axis) = 0 give W = (-(sin 0 cos 0), -sin 0,
    -(cos 0 cos 0)) = (-0, -0, -1), U = up x W, V = W x U, in float arithmetic (signed zeros kept)."""
    zero, one = F(0.0), F(1.0)
    sy, cy, sp, cp = F(0.0), F(1.0), F(0.0), F(1.0)  # sin/cos of yaw and pitch 0
    w = np.array([-(sy * cp), -sp, -(cy * cp)], F)
    w = (w * (one / np.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]))).astype(F)
    up = (zero, one, zero)
    u0 = np.array([up[1] * w[2] - up[2] * w[1], up[2] * w[0] - up[0] * w[2], up[0] * w[1] - up[1] * w[0]], F)
    u = (u0 * (one / np.sqrt(u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]))).astype(F)
    v0 = np.array([w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2], w[0] * u[1] - w[1] * u[0]], F)
    v = (v0 * (one / np.sqrt(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]))).astype(F)
    return u, v, w


class _Scene:
    """A SceneBuilder with the reference's helpers (surfaces from texture triples, named colors)."""

    def __init__(self, name, directory):
        self.name = name
        self.dir = directory
        self.b = SceneBuilder()
        self.eye = (55.0, 42.0, 155.6)

    def black(self):
        return self.b.constant(*BLACK)

    def const(self, c):
        return self.b.constant(*c)

    def surface(self, material, albedo, emission=None, normal=None, noise_amount=0.0, noise_scale=0.0):
        return self.b.surface(material, albedo, self.black() if emission is None else emission,
                              self.black() if normal is None else normal, noise_amount, noise_scale)

    def image(self, file, degrees, scale_u, scale_v):
        return self.b.image_file(_require(texture_path(self.dir, file)), degrees, scale_u, scale_v)

    def ground(self, surface):
        return self.b.primitive(self.b.plane(*GROUND), surface)

    def model(self, file, mapper, position=(0, 0, 0), scale=(1, 1, 1)):
        return _obj.load(self.b, _require(model_path(self.dir, file)), surface_mapper=mapper, position=position,
                         scale=scale)

    def compile(self):
        # The default camera: field of view 90 degrees at 800 x 800, focal distance 30, thin lens,
        # the eye of the scene, the basis of pitch 0 and yaw 0.
        e = self.eye
        self.b.camera(e, (e[0], e[1], e[2] - 1.0), 90.0, (800, 800), 0.0, 30.0)
        cs = self.b.compile(self.name)
        u, v, w = default_basis()
        cs.camera[7:10], cs.camera[10:13], cs.camera[13:16] = u, v, w
        return cs, SkyState()


def girl_scene(directory):
    """Scenes.java:106-152."""
    s = _Scene("Girl_Scene", directory)
    plane = s.surface(LAMBERTIAN, s.b.checkerboard(GRAY, WHITE, 0.0, 0.005, 0.005))
    fallback = s.surface(LAMBERTIAN, s.const(BLACK))
    table = {
        "01___Default": (LAMBERTIAN, rgb255(227, 161, 115)),
        "02___Default": (CLEAR_COAT, (0.8, 0.1, 0.8)),
        "03___Default": (CLEAR_COAT, rgb255(216, 192, 120)),
        "04___Default": (CLEAR_COAT, WHITE),
        "05___Default": (LAMBERTIAN, rgb255(227, 161, 115)),
    }
    surfaces = {k: s.surface(m, s.const(c)) for k, (m, c) in table.items()}
    s.ground(plane)
    s.model("aphroditegirl.obj", lambda g, m: surfaces.get(m, fallback), position=(0.0, 10.0, 0.0))
    return s.compile()


def house_scene(directory):
    """Scenes.java:154-228 (its model, "house interior.obj", is not among the reference's
    resources)."""
    s = _Scene("House_Scene", directory)
    plane_albedo = s.image("Texture_2.png", 0.0, 0.008, 0.008)
    fallback = s.surface(LAMBERTIAN, s.const(WHITE))
    table = {
        "floor_texture": (CLEAR_COAT, ("checker", GRAY, WHITE)),
        "wire_115115115": (PHONG, GRAY),
        "texture_1": (LAMBERTIAN, ("checker", RED, WHITE)),
        "texture_2": (LAMBERTIAN, ("checker", GREEN, WHITE)),
        "03___Default": (LAMBERTIAN, ("checker", BLUE, WHITE)),
        "crome": (LAMBERTIAN, GRAY),
        "table_wood_texture": (CLEAR_COAT, ORANGE),
        "sopha_wood_texture": (PHONG, ORANGE),
        "20___Default": (LAMBERTIAN, ORANGE),
        "double_sopha_wood_right_texture": (PHONG, GRAY),
    }

    def albedo(spec):
        if spec[0] == "checker":
            return s.b.checkerboard(spec[1], spec[2], 0.0, 5.0, 5.0)
        return s.const(spec)

    surfaces = {k: s.surface(m, albedo(c)) for k, (m, c) in table.items()}
    model = _require(model_path(directory, "house interior.obj"))
    s.ground(s.surface(LAMBERTIAN, plane_albedo))
    _obj.load(s.b, model, surface_mapper=lambda g, m: surfaces.get(m, fallback), position=(0.0, 10.0, 0.0))
    return s.compile()


def _rect(kind, a0, b0, a1, b1, c):
    """doCreateRectangleXY/XZ/YZ (Scenes.java:931-1014): two triangles over [min, max] of the two
    free axes at the fixed coordinate c, uv (0,0) (0,1) (1,1) and (0,0) (1,1) (1,0), each triangle's
    flat normal normalNormalized(a, b, c) and tangents from OrthoNormalBasis33F(normal).u."""
    lo0, hi0 = (a0, a1) if F(a0) <= F(a1) else (a1, a0)
    lo1, hi1 = (b0, b1) if F(b0) <= F(b1) else (b1, b0)

    def p(u, v):
        if kind == "XY":
            return (u, v, c)
        if kind == "XZ":
            return (u, c, v)
        return (c, u, v)  # YZ: (x, y, z) = (c, y, z)

    tri_a = [p(lo0, lo1), p(lo0, hi1), p(hi0, hi1)]
    tri_b = [p(lo0, lo1), p(hi0, hi1), p(hi0, lo1)]
    return [(tri_a, [(0.0, 0.0), (0.0, 1.0), (1.0, 1.0)]), (tri_b, [(0.0, 0.0), (1.0, 1.0), (1.0, 0.0)])]


def _normal_normalized(pa, pb, pc):
    a, b, c = (np.asarray(x, F) for x in (pa, pb, pc))
    e1, e2 = (b - a).astype(F), (c - a).astype(F)
    n = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]], F)
    ln = np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]).astype(F)
    return (n / ln).astype(F)


def _onb_u(w):
    """OrthoNormalBasis33F(w).u (Math4J): v from the smallest |component|, u = v x w."""
    w = np.asarray(w, F)
    w = (w / np.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]).astype(F)).astype(F)
    ax, ay, az = abs(w[0]), abs(w[1]), abs(w[2])
    if ax < ay and ax < az:
        v = np.array([F(0.0), w[2], -w[1]], F)
    elif ay < az:
        v = np.array([w[2], F(0.0), -w[0]], F)
    else:
        v = np.array([w[1], -w[0], F(0.0)], F)
    v = (v / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]).astype(F)).astype(F)
    return np.array([v[1] * w[2] - v[2] * w[1], v[2] * w[0] - v[0] * w[2], v[0] * w[1] - v[1] * w[0]], F)


def _rect_mesh(builder, rects):
    """A TriangleMesh from the rectangles' triangles, in order."""
    pos, nrm, uvs, tng = [], [], [], []
    for tri, uv in rects:
        n = _normal_normalized(*tri)
        t = _onb_u(n)
        for k in range(3):
            pos.append(tri[k])
            nrm.append(n)
            uvs.append(uv[k])
            tng.append(t)
    idx = np.arange(len(pos), dtype=np.int32).reshape(-1, 3)
    return builder.mesh(np.asarray(pos, F), idx, np.asarray(nrm, F), np.asarray(uvs, F), np.asarray(tng, F))


def house2_scene(directory):
    """Scenes.java:230-300."""
    s = _Scene("House_2_Scene", directory)
    floor = s.surface(LAMBERTIAN, s.b.checkerboard(GRAY, WHITE, 0.0, 5.0, 5.0))
    ground = s.surface(LAMBERTIAN, s.image("Texture_2.png", 0.0, 0.008, 0.008))
    roof = s.surface(LAMBERTIAN, s.const(WHITE))
    wall = s.surface(LAMBERTIAN, s.const(WHITE))
    k = F(0.1)

    def sc(*v):
        return [float(F(x) * k) for x in v]

    floor_r = _rect("XZ", *sc(0, 0, 500, 500, 0.2))
    roof_r = _rect("XZ", *sc(0, 0, 500, 500, 200))
    walls = [("XY", (0, 0, 500, 50, 0)), ("XY", (0, 50, 100, 150, 0)), ("XY", (400, 50, 500, 150, 0)),
             ("XY", (0, 150, 500, 200, 0)), ("XY", (0, 0, 500, 50, 500)), ("XY", (0, 50, 200, 100, 500)),
             ("XY", (300, 50, 500, 100, 500)), ("XY", (0, 100, 500, 200, 500)), ("YZ", (0, 0, 50, 500, 0)),
             ("YZ", (50, 0, 100, 200, 0)), ("YZ", (50, 300, 100, 500, 0)), ("YZ", (100, 0, 200, 500, 0)),
             ("YZ", (0, 0, 50, 500, 500)), ("YZ", (50, 0, 100, 200, 500)), ("YZ", (50, 300, 100, 500, 500)),
             ("YZ", (100, 0, 200, 500, 500))]
    wall_r = [t for kind, v in walls for t in _rect(kind, *sc(*v))]
    s.b.primitive(_rect_mesh(s.b, floor_r), floor)
    s.ground(ground)
    s.b.primitive(_rect_mesh(s.b, roof_r), roof)
    s.b.primitive(_rect_mesh(s.b, wall_r), wall)
    return s.compile()


def image_scene(directory):
    """Scenes.java:302-317."""
    s = _Scene("Image_Scene", directory)
    fbm = s.b.fbm((0.05, 0.05, 0.05), WHITE, 0.25, 0.5, 16)
    albedo = s.b.blend(fbm, s.const((0.5, 0.1, 0.5)), 0.75)
    monkey = s.surface(PHONG, albedo)
    ground = s.surface(LAMBERTIAN, s.const(GRAY))
    s.ground(ground)
    s.model("smoothMonkey2.obj", lambda g, m: monkey, position=(0.0, 100.0, 0.0), scale=(100.0, 100.0, 100.0))
    s.eye = (-8.75, 42.0, 332.6)
    return s.compile()


def material_showcase_scene(directory):
    """Scenes.java:319-408: a gray ground plane and 15 spheres of radius 16.5 at (x, 16.5, 20)."""
    s = _Scene("Material_Showcase_Scene", directory)
    b = s.b
    ground = s.surface(LAMBERTIAN, s.const(GRAY))
    spheres = [
        (40, CLEAR_COAT, lambda: s.const(GRAY), None, 0.0, 0.0),
        (80, GLASS, lambda: s.const(GRAY), None, 0.0, 0.0),
        (120, LAMBERTIAN, lambda: s.const(GRAY), None, 0.0, 0.0),
        (160, REFLECTION, lambda: s.const(GRAY), None, 0.0, 0.0),
        (200, PHONG, lambda: s.const(GRAY), None, 0.0, 0.0),
        (280, LAMBERTIAN, lambda: b.checkerboard(GRAY, WHITE, 0.0, 5.0, 5.0), None, 0.0, 0.0),
        (320, LAMBERTIAN, lambda: s.const(RED), None, 0.0, 0.0),
        (360, LAMBERTIAN, lambda: b.fbm((0.5, 0.05, 0.05), WHITE, 0.8, 0.5, 16), None, 0.0, 0.0),
        (400, LAMBERTIAN, lambda: s.image("Texture_2.png", 0.0, 1.0, 1.0), None, 0.0, 0.0),
        (440, LAMBERTIAN, lambda: b.surface_normal_texture(False), None, 0.0, 0.0),
        (480, LAMBERTIAN, lambda: b.blend(b.fbm((0.05, 0.05, 0.05), WHITE, 0.5, 0.5, 16),
                                          b.checkerboard(GRAY, RED, 0.0, 5.0, 5.0), 0.5), None, 0.0, 0.0),
        (520, LAMBERTIAN, lambda: b.uv_texture(), None, 0.0, 0.0),
        (560, LAMBERTIAN, lambda: b.bullseye((1.0, 0.1, 0.1), (0.1, 1.0, 0.1)), None, 0.0, 0.0),
        (640, REFLECTION, lambda: s.const(GRAY), lambda: s.image("bricks2_normal.jpg", 0.0, 4.0, 4.0), 0.0, 0.0),
        (680, GLASS, lambda: s.const(WHITE), None, 1.0, 16.0),
    ]
    surfaces = []
    for x, material, albedo, normal, amount, scale in spheres:
        surfaces.append((x, s.surface(material, albedo(), None, normal() if normal else None, amount, scale)))
    s.ground(ground)
    for x, surf in surfaces:
        b.primitive(b.sphere((0.0, 0.0, 0.0), 16.5), surf, position=(float(x), 16.5, 20.0))
    s.eye = (295.0, 42.0, 332.6)
    return s.compile()


def monkey_scene(directory):
    """Scenes.java:410-426."""
    s = _Scene("Monkey_Scene", directory)
    monkey = s.surface(PHONG, s.b.fbm((0.5, 0.05, 0.05), WHITE, 0.1, 0.5, 16))
    ground = s.surface(REFLECTION, s.const(tuple(float(F(v) / F(255.0)) for v in (135.0, 206.0, 235.0))), None, None, 1.0, 4.0)
    s.ground(ground)
    s.model("smoothMonkey2.obj", lambda g, m: monkey, position=(10.0, 100.0, 10.0))
    return s.compile()


def terrain_scene(directory):
    """Scenes.java:428-439."""
    s = _Scene("Terrain_Scene", directory)
    surf = s.surface(LAMBERTIAN, s.image("Texture_2.png", 0.0, 2.5, 2.5))
    s.b.primitive(s.b.terrain(8.0, 0.5, 0.0, 1.0, 8), surf)
    return s.compile()


def wine_glass_scene(directory):
    """Scenes.java:441-461."""
    s = _Scene("Wine_Glass_Scene", directory)
    ground = s.surface(LAMBERTIAN, s.b.checkerboard(GRAY, WHITE, 0.0, 0.1, 0.1))
    glass = s.surface(GLASS, s.const(GRAY))
    s.ground(ground)
    s.model("Wine_Glass.OBJ", lambda g, m: glass, position=(0.0, 39.0, 0.0), scale=(50.0, 50.0, 50.0))
    s.eye = (0.0, 42.0, 70.0)
    return s.compile()


def zealot_scene(directory):
    """Scenes.java:463-481 (its model and two of its textures are not among the reference's
    resources)."""
    s = _Scene("Zealot_Scene", directory)
    albedo = s.image("Zealot_albedo.png", 0.0, 1.0, 1.0)
    emission = s.image("Zealot_emissive.png", 0.0, 1.0, 1.0)
    normal = s.image("Zealot_normal.png", 0.0, 1.0, 1.0)
    zealot = s.surface(PHONG, albedo, emission, normal)
    ground = s.surface(LAMBERTIAN, s.const(GRAY))
    s.ground(ground)
    s.model("Zealot.obj", lambda g, m: zealot)
    s.eye = (0.0, 42.0, 70.0)
    return s.compile()


_BY_NAME = {
    "Girl_Scene": girl_scene,
    "House_Scene": house_scene,
    "House_2_Scene": house2_scene,
    "Image_Scene": image_scene,
    "Material_Showcase_Scene": material_showcase_scene,
    "Monkey_Scene": monkey_scene,
    "Terrain_Scene": terrain_scene,
    "Wine_Glass_Scene": wine_glass_scene,
    "Zealot_Scene": zealot_scene,
}


def scene_by_name(directory, name, resolution=None) -> tuple[CompiledScene, SkyState]:
    """Scenes.getSceneByName: unknown names build the material showcase. `resolution` (width,
    height) sets the camera to the size the scene is rendered at, as the application does
    (DayflowerApplication.java:334); without it the camera keeps the default 800 x 800."""
    cs, sky = _BY_NAME.get(name, material_showcase_scene)(directory)
    if resolution is not None:
        camera_set_resolution(cs.camera, *resolution)
    return cs, sky
