"""Seeded synthetic scenes with the shapes, sizes and value distributions of the benchmark configs.

The reference publishes no benchmark scenes, so each workload is generated from a seed:
  sphere_scene      - ground plane (checkerboard, Lambertian) + 3 unit spheres (Lambertian, Glass,
                      ClearCoat), Perez sky T=2, sun at 45 degrees; 512x512, depth 5, RR 3, Reinhard.
  mesh_scene        - an fBm-displaced geodesic icosphere (frequency 100: 200,000 triangles) in four
                      Lambertian/Phong regions (Phong exponent U(10,200) per region, extension
                      records) over a 512x512 fBm heightfield (522,242 triangles); 1920x1080,
                      depth 8, ACES.
  instances_scene   - 40 displaced icospheres of 50,000 triangles each (2M), scale U(0.5,3) in a
                      100^3 box, Glass/Reflection/Lambertian, 500 emissive triangle primitives with
                      emission U(1,20) (extension records).
  spheres_on_plane  - 256 spheres on a plane under a Perez sky (the inverse-rendering scene).
  batch_workload    - 64 scenes (displaced icosphere on a plane) with log-uniform triangle counts in
                      [1k, 500k], resolutions {256^2, 512^2, 1024^2}, spp {16, 64, 256}.
Geometry uses only IEEE arithmetic (+, -, *, /, sqrt, floor) so a seed gives the same arrays on
every host; noise is the reference's simplex fBm (AbstractKernel.java:695-716, 762-900).
"""
from __future__ import annotations

import numpy as np

from . import scene as sc
from .noise_tables import PERMUTATION

PERM = np.asarray(PERMUTATION + PERMUTATION, dtype=np.int64)
PERM12 = PERM % 12
GRAD3 = np.asarray([1, 1, 0, -1, 1, 0, 1, -1, 0, -1, -1, 0, 1, 0, 1, -1, 0, 1, 1, 0, -1, -1, 0, -1,
                    0, 1, 1, 0, -1, 1, 0, 1, -1, 0, -1, -1], dtype=np.float32).reshape(12, 3)


def _ffloor(v):
    i = v.astype(np.int64)
    return np.where(v < i, i - 1, i)


def simplex3(x, y, z):
    """Vectorised simplexNoiseXYZ (AbstractKernel.java:812-900), float32 arithmetic."""
    f32 = np.float32
    x, y, z = (np.asarray(a, dtype=np.float32) for a in (x, y, z))
    F3, G3 = f32(1.0 / 3.0), f32(1.0 / 6.0)
    s = (x + y + z) * F3
    i, j, k = _ffloor(x + s), _ffloor(y + s), _ffloor(z + s)
    t = (i + j + k).astype(np.float32) * G3
    x0 = x - (i.astype(np.float32) - t)
    y0 = y - (j.astype(np.float32) - t)
    z0 = z - (k.astype(np.float32) - t)
    c1 = x0 >= y0
    c2 = y0 >= z0
    c3 = x0 >= z0
    # The branch structure of the reference, one mask per leaf.
    i1 = np.zeros_like(i); j1 = np.zeros_like(i); k1 = np.zeros_like(i)
    i2 = np.zeros_like(i); j2 = np.zeros_like(i); k2 = np.zeros_like(i)
    a = c1 & c2
    b = c1 & ~c2 & c3
    c = c1 & ~c2 & ~c3
    yz = y0 < z0
    xz = x0 < z0
    d = ~c1 & yz
    e = ~c1 & ~yz & xz
    g = ~c1 & ~yz & ~xz
    i1[a] = 1; i2[a] = 1; j2[a] = 1
    i1[b] = 1; i2[b] = 1; k2[b] = 1
    k1[c] = 1; i2[c] = 1; k2[c] = 1
    k1[d] = 1; j2[d] = 1; k2[d] = 1
    j1[e] = 1; j2[e] = 1; k2[e] = 1
    j1[g] = 1; i2[g] = 1; j2[g] = 1
    x1 = x0 - i1.astype(np.float32) + G3
    y1 = y0 - j1.astype(np.float32) + G3
    z1 = z0 - k1.astype(np.float32) + G3
    x2 = x0 - i2.astype(np.float32) + f32(2.0) * G3
    y2 = y0 - j2.astype(np.float32) + f32(2.0) * G3
    z2 = z0 - k2.astype(np.float32) + f32(2.0) * G3
    x3 = x0 - f32(1.0) + f32(3.0) * G3
    y3 = y0 - f32(1.0) + f32(3.0) * G3
    z3 = z0 - f32(1.0) + f32(3.0) * G3
    ii, jj, kk = i & 0xFF, j & 0xFF, k & 0xFF
    gi0 = PERM12[ii + PERM[jj + PERM[kk]]]
    gi1 = PERM12[ii + i1 + PERM[jj + j1 + PERM[kk + k1]]]
    gi2 = PERM12[ii + i2 + PERM[jj + j2 + PERM[kk + k2]]]
    gi3 = PERM12[ii + 1 + PERM[jj + 1 + PERM[kk + 1]]]

    def corner(tx, ty, tz, gi):
        tt = f32(0.6) - tx * tx - ty * ty - tz * tz
        gg = GRAD3[gi]
        dot = gg[..., 0] * tx + gg[..., 1] * ty + gg[..., 2] * tz
        return np.where(tt < 0, f32(0.0), (tt * tt) * (tt * tt) * dot).astype(np.float32)

    n = corner(x0, y0, z0, gi0) + corner(x1, y1, z1, gi1) + corner(x2, y2, z2, gi2) + corner(x3, y3, z3, gi3)
    return (f32(32.0) * n).astype(np.float32)


def fbm3(frequency, gain, minimum, maximum, octaves, x, y, z):
    """simplexFractionalBrownianMotionXYZ (AbstractKernel.java:695-716)."""
    f32 = np.float32
    amp, max_amp, freq = f32(1.0), f32(0.0), f32(frequency)
    noise = np.zeros(np.shape(x), dtype=np.float32)
    for _ in range(int(octaves)):
        noise = noise + simplex3(x * freq, y * freq, z * freq) * amp
        max_amp = f32(max_amp + amp)
        amp = f32(amp * f32(gain))
        freq = f32(freq * f32(2.0))
    noise = noise / max_amp
    return (noise * (f32(maximum) - f32(minimum)) / f32(2.0) + (f32(maximum) + f32(minimum)) / f32(2.0)).astype(np.float32)


# -----------------------------------------------------------------------------------------------
# Geometry.

def geodesic_sphere(frequency: int):
    """Unit geodesic icosphere: each icosahedron face split into frequency^2 triangles.

    Returns (positions float64 [V,3], indices int32 [F,3], face_region int [F] = base face id)."""
    t = (1.0 + np.sqrt(5.0)) / 2.0
    base = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                     [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                      [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                      [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    n = int(frequency)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = (ii + jj) <= n
    ii, jj = ii[keep], jj[keep]
    lut = -np.ones((n + 1, n + 1), dtype=np.int64)
    lut[ii, jj] = np.arange(len(ii))
    # Local triangles of one face.
    tri = []
    for i in range(n):
        for j in range(n - i):
            tri.append((lut[i, j], lut[i + 1, j], lut[i, j + 1]))
            if i + j < n - 1:
                tri.append((lut[i + 1, j], lut[i + 1, j + 1], lut[i, j + 1]))
    tri = np.asarray(tri, dtype=np.int64)
    pts, idx, region = [], [], []
    nloc = len(ii)
    for f, (a, b, c) in enumerate(faces):
        A, B, Cc = base[a], base[b], base[c]
        p = A[None, :] + (B - A)[None, :] * (ii[:, None] / n) + (Cc - A)[None, :] * (jj[:, None] / n)
        pts.append(p)
        idx.append(tri + f * nloc)
        region.append(np.full(len(tri), f))
    pts = np.concatenate(pts)
    pts /= np.sqrt((pts * pts).sum(1))[:, None]
    idx = np.concatenate(idx)
    region = np.concatenate(region)
    # Merge the vertices shared by neighbouring faces.
    key = np.round(pts * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)
    remap = np.empty_like(order)
    remap[order] = np.arange(len(order))
    pts = pts[first[order]]
    idx = remap[inv.reshape(-1)[idx]]
    return pts, idx.astype(np.int32), region


def vertex_normals(pos, idx):
    p = pos.astype(np.float64)
    a, b, c = p[idx[:, 0]], p[idx[:, 1]], p[idx[:, 2]]
    fn = np.cross(b - a, c - a)
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, idx[:, k], fn)
    n /= np.maximum(np.sqrt((n * n).sum(1)), 1e-30)[:, None]
    return n


def tangents_for(normals):
    up = np.where(np.abs(normals[:, 1:2]) < 0.999, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(up, normals)
    t /= np.maximum(np.sqrt((t * t).sum(1)), 1e-30)[:, None]
    return t


def displaced_icosphere(frequency: int, amplitude: float, seed: int, radius: float = 1.0):
    pos, idx, region = geodesic_sphere(frequency)
    off = np.float32((seed * 7919) % 1000) * np.float32(0.731)
    x = (pos[:, 0] * 2.0).astype(np.float32) + off
    y = (pos[:, 1] * 2.0).astype(np.float32)
    z = (pos[:, 2] * 2.0).astype(np.float32)
    h = fbm3(1.0, 0.5, -1.0, 1.0, 6, x, y, z).astype(np.float64)
    pos = pos * (radius + amplitude * h)[:, None]
    nrm = vertex_normals(pos, idx)
    uv = np.stack([0.5 + 0.5 * pos[:, 0] / (radius + amplitude), 0.5 + 0.5 * pos[:, 1] / (radius + amplitude)], 1)
    return pos, idx, region, nrm, uv


def heightfield(n: int, size: float, height: float, seed: int, octaves: int = 6):
    xs = np.linspace(-size / 2, size / 2, n)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    off = np.float32((seed * 104729) % 1000) * np.float32(0.377)
    h = fbm3(0.05, 0.5, -1.0, 1.0, octaves, X.astype(np.float32) + off, np.zeros_like(X, dtype=np.float32),
             Z.astype(np.float32)).astype(np.float64)
    pos = np.stack([X, h * height, Z], -1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    v00 = (i * n + j).ravel()
    v10 = ((i + 1) * n + j).ravel()
    v01 = (i * n + j + 1).ravel()
    v11 = ((i + 1) * n + j + 1).ravel()
    idx = np.concatenate([np.stack([v00, v01, v10], 1), np.stack([v10, v01, v11], 1)]).astype(np.int32)
    nrm = vertex_normals(pos, idx)
    uv = np.stack([(X.ravel() + size / 2) / size, (Z.ravel() + size / 2) / size], 1)
    return pos, idx, nrm, uv


# -----------------------------------------------------------------------------------------------
# Workloads. Each returns (CompiledScene, SkyState, params dict, (width, height)).

SUN_45 = (0.5, 0.70710677, 0.5)  # elevation 45 degrees (azimuth 45)


def sphere_scene(seed: int = 0, width: int = 512, height: int = 512, checker_colors=((0.5, 0.5, 0.5), (0.5, 0.5, 0.5))):
    """`checker_colors`: the ground's two checkerboard colours; the default is the reference's
    CheckerboardTexture() (GRAY and GRAY, CheckerboardTexture.java:109-110), parity tests pass two."""
    rng = np.random.default_rng(seed)
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    checker = b.checkerboard(checker_colors[0], checker_colors[1], 0.0, 5.0, 5.0)
    ground = b.surface(sc.LAMBERTIAN, checker, black, black)
    b.primitive(b.plane((0, 0, 0), (0, 0, 1), (1, 0, 0)), ground)
    sphere = b.sphere((0, 0, 0), 1.0)
    albedo = rng.uniform(0.2, 0.9, 3)
    mats = [(sc.LAMBERTIAN, b.constant(*albedo)), (sc.GLASS, b.constant(1, 1, 1)),
            (sc.CLEAR_COAT, b.constant(*rng.uniform(0.2, 0.9, 3)))]
    for mat, tex in mats:
        x, z = rng.uniform(-4, 4, 2)
        b.primitive(sphere, b.surface(mat, tex, black, black), position=(float(x), 1.0, float(z)))
    b.camera((0, 2, 10), (0, 0, 0), 90.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3, tone_mapper_type=2,
                  tone_mapper_exposure=1.0)
    return b.compile("sphere_scene"), sc.SkyState(SUN_45, 2.0), params, (width, height)


def mesh_scene(seed: int = 1, width: int = 1920, height: int = 1080, frequency: int = 100, grid: int = 512):
    rng = np.random.default_rng(seed)
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    pos, idx, region, nrm, uv = displaced_icosphere(frequency, 0.1, seed, radius=3.0)
    pos = pos + np.array([0.0, 4.0, 0.0])
    tng = tangents_for(nrm)
    # Four regions by base face id: Lambertian and Phong alternate; each Phong region has its own
    # exponent U(10, 200) (an extension record: the reference's compiler drops the exponent).
    quadrant = region % 4
    rng_x = np.random.default_rng(seed + 7919)
    for q in range(4):
        sel = idx[quadrant == q]
        mat = sc.LAMBERTIAN if q % 2 == 0 else sc.PHONG
        surf = b.surface(mat, b.constant(*rng.uniform(0.3, 0.9, 3)), black, black)
        b.primitive(b.mesh(pos, sel, nrm, uv, tng), surf,
                    phong_exponent=float(rng_x.uniform(10.0, 200.0)) if mat == sc.PHONG else None)
    hp, hi, hn, huv = heightfield(grid, 60.0, 2.0, seed)
    b.primitive(b.mesh(hp, hi, hn, huv, tangents_for(hn)), b.surface(sc.LAMBERTIAN, b.constant(0.55, 0.5, 0.45), black, black))
    b.camera((0, 6, 14), (0, 3.5, 0), 70.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=8, pt_ray_depth_russian_roulette=5, tone_mapper_type=1,
                  tone_mapper_exposure=1.0)
    return b.compile("mesh_scene"), sc.SkyState(SUN_45, 2.0), params, (width, height)


def small_mesh_scene(seed: int = 3, width: int = 96, height: int = 64, frequency: int = 8, grid: int = 24):
    """mesh_scene's structure at test sizes (planes, spheres, meshes, transforms)."""
    rng = np.random.default_rng(seed)
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    pos, idx, region, nrm, uv = displaced_icosphere(frequency, 0.1, seed, radius=1.5)
    tng = tangents_for(nrm)
    for q in range(2):
        sel = idx[region % 2 == q]
        mat = sc.LAMBERTIAN if q == 0 else sc.PHONG
        surf = b.surface(mat, b.constant(*rng.uniform(0.3, 0.9, 3)), black, black)
        b.primitive(b.mesh(pos, sel, nrm, uv, tng), surf, position=(0.0, 2.0, 0.0), scale=(1.0, 1.2, 1.0))
    hp, hi, hn, huv = heightfield(grid, 20.0, 1.0, seed)
    b.primitive(b.mesh(hp, hi, hn, huv, tangents_for(hn)), b.surface(sc.LAMBERTIAN, b.constant(0.5, 0.5, 0.45), black, black))
    b.primitive(b.sphere((0, 0, 0), 0.7), b.surface(sc.GLASS, b.constant(1, 1, 1), black, black), position=(2.5, 1.5, 1.0))
    b.primitive(b.sphere((0, 0, 0), 0.6), b.surface(sc.REFLECTION, b.constant(0.9, 0.9, 0.9), black, black), position=(-2.5, 1.2, 0.5))
    b.primitive(b.sphere((0, 0, 0), 0.5), b.surface(sc.CLEAR_COAT, b.constant(0.8, 0.2, 0.2), black, black), position=(0.0, 0.8, 3.0))
    b.camera((0, 4, 10), (0, 1.5, 0), 60.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=6, pt_ray_depth_russian_roulette=3, tone_mapper_type=1,
                  tone_mapper_exposure=1.0)
    return b.compile("small_mesh_scene"), sc.SkyState(SUN_45, 2.0), params, (width, height)


def instances_scene(seed: int = 2, width: int = 1920, height: int = 1080, frequency: int = 50, count: int = 40,
                    lights: int = 500):
    rng = np.random.default_rng(seed)
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    mats = [sc.GLASS, sc.REFLECTION, sc.LAMBERTIAN]
    for k in range(count):
        pos, idx, region, nrm, uv = displaced_icosphere(frequency, 0.1, seed * 1000 + k)
        s = float(rng.uniform(0.5, 3.0))
        c = rng.uniform(0.0, 100.0, 3)
        mat = mats[k % 3]
        surf = b.surface(mat, b.constant(*rng.uniform(0.3, 0.95, 3)), black, black)
        b.primitive(b.mesh(pos * s + c, idx, nrm, uv, tangents_for(nrm)), surf)
    # Area lights: `lights` triangle primitives with a white emission texture scaled by U(1, 20) each
    # (an extension record: the reference packs emission into 8 bits clamped to 1).
    lp = rng.uniform(0.0, 100.0, (lights, 3))
    tris = []
    for k in range(lights):
        a = lp[k]
        tris.append([a, a + rng.normal(0, 1.0, 3), a + rng.normal(0, 1.0, 3)])
    tris = np.asarray(tris).reshape(-1, 3)
    tidx = np.arange(len(tris), dtype=np.int32).reshape(-1, 3)
    n = vertex_normals(tris, tidx)
    tg = tangents_for(n)
    emit = b.surface(sc.LAMBERTIAN, b.constant(1, 1, 1), b.constant(1, 1, 1), black)
    scale = np.random.default_rng(seed + 104729).uniform(1.0, 20.0, lights)
    zero_uv = np.zeros((3, 2))
    for k in range(lights):
        v = slice(3 * k, 3 * k + 3)
        b.primitive(b.mesh(tris[v], [[0, 1, 2]], n[v], zero_uv, tg[v], as_mesh=False), emit, emission_scale=float(scale[k]))
    b.camera((50, 50, -60), (50, 50, 50), 70.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3, tone_mapper_type=1,
                  tone_mapper_exposure=1.0)
    return b.compile("instances_scene"), sc.SkyState(SUN_45, 2.0), params, (width, height)


def spheres_on_plane(seed: int = 4, width: int = 512, height: int = 512, count: int = 256, albedo=None):
    rng = np.random.default_rng(seed)
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    ground = b.surface(sc.LAMBERTIAN, b.constant(0.5, 0.5, 0.5), black, black)
    b.primitive(b.plane((0, 0, 0), (0, 0, 1), (1, 0, 0)), ground)
    sphere = b.sphere((0, 0, 0), 0.4)
    side = int(np.ceil(np.sqrt(count)))
    alb = rng.uniform(0.1, 0.9, (count, 3)) if albedo is None else np.asarray(albedo).reshape(count, 3)
    for k in range(count):
        x = (k % side - side / 2) * 1.0 + 0.5
        z = (k // side - side / 2) * 1.0 + 0.5
        b.primitive(sphere, b.surface(sc.LAMBERTIAN, b.constant(*alb[k]), black, black), position=(x, 0.4, z))
    b.camera((0, 9, 14), (0, 0, 0), 70.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3, tone_mapper_type=2,
                  tone_mapper_exposure=1.0)
    return b.compile("spheres_on_plane"), sc.SkyState(SUN_45, 3.0), params, (width, height)


def batch_scene(seed: int, triangles: int, width: int, height: int, threads: int = 0):
    """One scene of the batched workload: an fBm-displaced icosphere with about `triangles`
    triangles (20 f^2 for frequency f) in Lambertian/Phong/Glass regions on a checkerboard plane,
    Perez sky with a seeded turbidity and sun; depth 5, Russian roulette from 3, Reinhard."""
    rng = np.random.default_rng(1000 + seed)
    f = max(1, int(round(np.sqrt(triangles / 20.0))))
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    checker = b.checkerboard((0.5, 0.5, 0.5), (0.2, 0.2, 0.2), 0.0, 5.0, 5.0)
    b.primitive(b.plane((0, 0, 0), (0, 0, 1), (1, 0, 0)), b.surface(sc.LAMBERTIAN, checker, black, black))
    pos, idx, region, nrm, uv = displaced_icosphere(f, 0.1, seed, radius=1.5)
    pos = pos + np.array([0.0, 1.6, 0.0])
    tng = tangents_for(nrm)
    mats = (sc.LAMBERTIAN, sc.PHONG, sc.GLASS)
    for q in range(3):
        sel = idx[region % 3 == q]
        if len(sel) == 0:
            continue
        tex = b.constant(1, 1, 1) if mats[q] == sc.GLASS else b.constant(*rng.uniform(0.2, 0.9, 3))
        b.primitive(b.mesh(pos, sel, nrm, uv, tng), b.surface(mats[q], tex, black, black))
    az = float(rng.uniform(0, 2 * np.pi))
    el = float(rng.uniform(0.35, 1.2))
    sun = (float(np.cos(el) * np.cos(az)), float(np.sin(el)), float(np.cos(el) * np.sin(az)))
    b.camera((0, 2.5, 6), (0, 1.4, 0), 70.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3, tone_mapper_type=2,
                  tone_mapper_exposure=1.0, seed=seed)
    return b.compile(f"batch_scene_{seed}", threads=threads), sc.SkyState(sun, float(rng.uniform(2.0, 4.0))), params


def batch_workload(seed: int = 5, count: int = 64, tri_range=(1000, 500000), resolutions=(256, 512, 1024),
                   spps=(16, 64, 256)):
    """The batched-rendering workload: `count` seeded scenes, triangle counts log-uniform in
    `tri_range`, square resolutions and samples per pixel drawn uniformly from the lists.
    Returns a list of dicts {scene, sky, params, width, height, spp, triangles}."""
    rng = np.random.default_rng(seed)
    tris = np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]), count))
    res = rng.choice(resolutions, count)
    spp = rng.choice(spps, count)
    out = []
    for i in range(count):
        cs, sky, params = batch_scene(seed * 1000 + i, int(tris[i]), int(res[i]), int(res[i]))
        out.append(dict(scene=cs, sky=sky, params=params, width=int(res[i]), height=int(res[i]), spp=int(spp[i]),
                        triangles=int(cs.triangles.size // 12)))
    return out


def inverse_scene(seed: int = 6, width: int = 512, height: int = 512, count: int = 256, phong_every: int = 4,
                  plane: bool = True):
    """The inverse-rendering workload: `count` spheres (radius 0.4) on a grid over a Lambertian
    plane under a Perez sky, every `phong_every`-th sphere Phong, the rest Lambertian. Sphere
    albedo textures are white, so the per-primitive albedo parameter is the albedo. Returns
    (scene, params, (width, height), truth, start): truth/start hold per-primitive albedo (P, 3),
    Phong exponents (P,), turbidity and sun direction - ground truth albedo U(0.1, 0.9)^3 and
    turbidity 3, start albedo 0.5 and turbidity 2 (the plane, primitive 0, keeps multiplier 1)."""
    rng = np.random.default_rng(seed)
    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    white = b.constant(1, 1, 1)
    if plane:
        b.primitive(b.plane((0, 0, 0), (0, 0, 1), (1, 0, 0)), b.surface(sc.LAMBERTIAN, b.constant(0.5, 0.5, 0.5), black, black))
    sphere = b.sphere((0, 0, 0), 0.4)
    side = int(np.ceil(np.sqrt(count)))
    lam = b.surface(sc.LAMBERTIAN, white, black, black)
    pho = b.surface(sc.PHONG, white, black, black)
    spacing = 1.0 if count > 16 else 1.6
    for k in range(count):
        x = (k % side - (side - 1) / 2) * spacing
        z = (k // side - (side - 1) / 2) * spacing
        b.primitive(sphere, pho if phong_every and k % phong_every == phong_every - 1 else lam, position=(x, 0.4, z))
    dist = 1.1 * side * spacing
    b.camera((0, 0.65 * dist, dist), (0, 0, 0), 60.0, (width, height))
    params = dict(renderer_type=2, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3, tone_mapper_type=2,
                  tone_mapper_exposure=1.0)
    n = count + (1 if plane else 0)
    off = 1 if plane else 0
    truth_albedo = np.ones((n, 3), np.float32)
    truth_albedo[off:] = rng.uniform(0.1, 0.9, (count, 3))
    exponent = np.full(n, 50.0, np.float32)
    exponent[off:] = rng.uniform(10.0, 200.0, count)
    sun = tuple(float(v) for v in SUN_45)
    truth = dict(albedo=truth_albedo, phong_exponent=exponent, turbidity=3.0, sun_direction=sun)
    start_albedo = np.ones((n, 3), np.float32)
    start_albedo[off:] = 0.5
    start = dict(albedo=start_albedo, phong_exponent=exponent.copy(), turbidity=2.0, sun_direction=sun)
    return b.compile("inverse_scene"), params, (width, height), truth, start
