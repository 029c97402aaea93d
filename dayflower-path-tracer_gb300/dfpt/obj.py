"""Wavefront OBJ loader for SceneBuilder: ObjectLoader.load restated
(src/main/java/org/dayflower/pathtracer/scene/wavefront/ObjectLoader.java:118-194, 351-637).

What it reproduces, with Java float arithmetic (float32, one rounding per operation):
  * lines split on single spaces; `g` sets the group, `usemtl` the material, `v`, `vt`, `vn` the
    attribute lists; `f` faces are fan-triangulated (1, 2+i, 3+i); other lines are ignored;
  * face tokens `v[/vt[/vn]]` are 1-based; a token without vt/vn keeps index 0 for them, and a file
    where any token carries vt (vn) uses texture coordinates (normals) for every token;
  * (v, vt, vn) triples become model vertices (first occurrence order), carrying the group and
    material of their first occurrence;
  * without `vn`, normals are computed per position index: the normalised face normal
    cross(p1 - p0, p2 - p0) summed over the faces in order, then normalised;
  * tangents are always computed per position index from the first occurrence's texture
    coordinate, with the reference's z component (it repeats the y expression), summed, normalised;
  * every triangle's texture coordinates are flipped to (u, 1 - v);
  * a new mesh primitive starts whenever the group of a triangle's first vertex changes, with the
    surface `surface_mapper(group, material)`;
  * files named aphroditegirl.obj or smoothMonkey2.obj are scaled by 100 (the reference's hack:
    positions by the scaling matrix, normals and tangents by the transpose of its inverse).
"""
from __future__ import annotations

import os
from fractions import Fraction

import numpy as np

F = np.float32


def _java_float(token: str) -> np.float32:
    """Float.valueOf: the decimal rounded once to the nearest float (optional f/F/d/D suffix)."""
    t = token.strip()
    if t and t[-1] in "fFdD" and not t.lower().endswith("infinity"):
        t = t[:-1]
    if t in ("NaN", "+NaN", "-NaN"):
        return F(np.nan)
    if t.lstrip("+-") == "Infinity":
        return F(-np.inf) if t.startswith("-") else F(np.inf)
    d = float(t)
    f = F(d)
    # Rounding through double is exact unless the double sits on a float midpoint.
    if np.isfinite(f) and d != 0.0:
        lo, hi = np.nextafter(f, F(-np.inf)), np.nextafter(f, F(np.inf))
        for other in (lo, hi):
            if (float(f) + float(other)) / 2.0 == d:
                exact = Fraction(t)
                a, b = Fraction(float(f)), Fraction(float(other))
                da, db = abs(exact - a), abs(exact - b)
                if db < da or (db == da and int(np.asarray(other).view(np.int32)) % 2 == 0):
                    f = other
                break
    return f


def _normalize(v):
    """Vector3F.normalize: divide by sqrt(x*x + y*y + z*z), all in float."""
    l2 = (v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2]
    with np.errstate(invalid="ignore", divide="ignore"):
        return (v / np.sqrt(l2.astype(np.float64)).astype(F)[..., None]).astype(F)


class ObjModel:
    """The parsed file (ObjectModel) and its indexed form (ObjectModel.toIndexedModel)."""

    def __init__(self, text: str):
        self.positions, self.uvs, self.normals = [], [], []
        self.faces = []  # (v, vt, vn) per corner, 3 per triangle
        self.face_groups, self.face_materials = [], []
        self.has_uv = self.has_normal = False
        group = material = ""
        for line in text.splitlines():
            tokens = [t for t in line.split(" ") if t != ""]
            if not tokens or tokens[0] == "#":
                continue
            key = tokens[0]
            if key == "g":
                group = tokens[1]
            elif key == "usemtl":
                material = tokens[1]
            elif key == "v":
                self.positions.append((_java_float(tokens[1]), _java_float(tokens[2]), _java_float(tokens[3])))
            elif key == "vt":
                self.uvs.append((_java_float(tokens[1]), _java_float(tokens[2])))
            elif key == "vn":
                self.normals.append((_java_float(tokens[1]), _java_float(tokens[2]), _java_float(tokens[3])))
            elif key == "f":
                for i in range(len(tokens) - 3):
                    for tok in (tokens[1], tokens[2 + i], tokens[3 + i]):
                        self.faces.append(self._index(tok))
                        self.face_groups.append(group)
                        self.face_materials.append(material)

    def _index(self, token: str):
        # Java's split drops trailing empty strings: "1/2/" is ["1", "2"].
        values = token.split("/")
        while len(values) > 1 and values[-1] == "":
            values.pop()
        v, vt, vn = int(values[0]) - 1, 0, 0
        if len(values) > 1:
            if values[1] != "":
                self.has_uv = True
                vt = int(values[1]) - 1
            if len(values) > 2:
                self.has_normal = True
                vn = int(values[2]) - 1
        return v, vt, vn

    def indexed(self):
        """Returns per model vertex: uv (n, 2), position (n, 3), normal (n, 3), tangent (n, 3),
        group, material lists, and the index triples (t, 3)."""
        key0, key1 = {}, {}
        uv0, pos0, nrm0, grp0, mat0, idx0 = [], [], [], [], [], []
        uv1, pos1, nrm1, idx1 = [], [], [], []
        m0_to_m1 = {}
        zero2, zero3 = (F(0), F(0)), (F(0), F(0), F(0))
        for i, (v, vt, vn) in enumerate(self.faces):
            uv = self.uvs[vt] if self.has_uv else zero2
            p = self.positions[v]
            nrm = self.normals[vn] if self.has_normal else zero3
            k0 = key0.get((v, vt, vn))
            if k0 is None:
                k0 = key0[(v, vt, vn)] = len(pos0)
                uv0.append(uv); pos0.append(p); grp0.append(self.face_groups[i]); mat0.append(self.face_materials[i])
                if self.has_normal:
                    nrm0.append(nrm)
            k1 = key1.get(v)
            if k1 is None:
                k1 = key1[v] = len(pos1)
                uv1.append(uv); pos1.append(p); nrm1.append(nrm)
            idx0.append(k0)
            idx1.append(k1)
            m0_to_m1[k0] = k1
        P1 = np.asarray(pos1, F).reshape(-1, 3)
        T1 = np.asarray(uv1, F).reshape(-1, 2)
        I1 = np.asarray(idx1, np.int64).reshape(-1, 3)
        map01 = np.asarray([m0_to_m1[i] for i in range(len(pos0))], np.int64)
        if not self.has_normal:
            N1 = np.asarray(nrm1, F).reshape(-1, 3).copy()
            e0 = P1[I1[:, 1]] - P1[I1[:, 0]]
            e1 = P1[I1[:, 2]] - P1[I1[:, 0]]
            fn = np.stack([e0[:, 1] * e1[:, 2] - e0[:, 2] * e1[:, 1], e0[:, 2] * e1[:, 0] - e0[:, 0] * e1[:, 2],
                           e0[:, 0] * e1[:, 1] - e0[:, 1] * e1[:, 0]], 1).astype(F)
            fn = _normalize(fn)
            # Summed in face order, corner 0, 1, 2 (np.add.at is sequential for repeated indices).
            np.add.at(N1, I1.reshape(-1), np.repeat(fn, 3, axis=0))
            N1 = _normalize(N1)
            N0 = N1[map01]
        else:
            N0 = np.asarray(nrm0, F).reshape(-1, 3)
        e0 = P1[I1[:, 1]] - P1[I1[:, 0]]
        e1 = P1[I1[:, 2]] - P1[I1[:, 0]]
        du0 = T1[I1[:, 1], 0] - T1[I1[:, 0], 0]
        dv0 = T1[I1[:, 1], 1] - T1[I1[:, 0], 1]
        du1 = T1[I1[:, 2], 0] - T1[I1[:, 0], 0]
        dv1 = T1[I1[:, 2], 1] - T1[I1[:, 0], 1]
        div = (du0 * dv1 - du1 * dv0).astype(F)
        # Float.compare(dividend, 0.0F) == 0 holds for +0.0 only.
        pos_zero = (div == 0) & ~np.signbit(div)
        with np.errstate(divide="ignore", invalid="ignore"):
            frac = np.where(pos_zero, F(0), (F(1) / div).astype(F)).astype(F)
            ty = (dv1 * e0[:, 1] - dv0 * e1[:, 1]).astype(F)
            tan = np.stack([frac * (dv1 * e0[:, 0] - dv0 * e1[:, 0]), frac * ty, frac * ty], 1).astype(F)
        T1n = np.zeros((len(pos1), 3), F)
        np.add.at(T1n, I1.reshape(-1), np.repeat(tan, 3, axis=0))
        T1n = _normalize(T1n)
        return (np.asarray(uv0, F).reshape(-1, 2), np.asarray(pos0, F).reshape(-1, 3), N0.astype(F), T1n[map01], grp0, mat0,
                np.asarray(idx0, np.int64).reshape(-1, 3))


def _scale_hack(pos, nrm, tng):
    """Triangle.transformToWorldSpace with Matrix44F.scaling(100) and its inverse (Math4J)."""
    s = F(100)
    # The inverse's diagonal as Matrix44F.inverse computes it: (s*s) * (1 / (s*s*s*1)).
    a, l = s * s, s * F(1)
    det = a * l
    r = F(1) / det
    inv = (s * l) * r
    inv3 = (s * s) * r  # element33 = (+e44 * a) * r with a = s*s
    inv_diag = np.array([inv, inv, inv3], F)
    z = F(0)
    p = np.stack([s * pos[:, 0] + z * pos[:, 1] + z * pos[:, 2] + z,
                  z * pos[:, 0] + s * pos[:, 1] + z * pos[:, 2] + z,
                  z * pos[:, 0] + z * pos[:, 1] + s * pos[:, 2] + z], 1).astype(F)

    def tt(v):
        return np.stack([inv_diag[0] * v[:, 0] + z * v[:, 1] + z * v[:, 2],
                         z * v[:, 0] + inv_diag[1] * v[:, 1] + z * v[:, 2],
                         z * v[:, 0] + z * v[:, 1] + inv_diag[2] * v[:, 2]], 1).astype(F)

    return p, tt(nrm), tt(tng)


def load(builder, source, surface=None, surface_mapper=None, position=(0, 0, 0), rotation=(0, 0, 0, 1), scale=(1, 1, 1),
         name=None):
    """Adds the model's primitives to `builder` and returns their indices. `source` is a path or the
    file's text (then `name` stands in for the file name). `surface_mapper(group, material)` returns
    a builder surface index; `surface` is the one surface for every group (the reference's default
    is Lambertian gray when neither is given)."""
    if isinstance(source, (str, os.PathLike)) and os.path.exists(str(source)):
        with open(source, "r", encoding="utf-8", errors="replace") as fh:
            text = fh.read()
        name = name or os.path.basename(str(source))
    else:
        text = str(source)
        name = name or ""
    if surface_mapper is None:
        if surface is None:
            gray = builder.constant(0.5, 0.5, 0.5)  # Color.GRAY
            black = builder.constant(0, 0, 0)
            surface = builder.surface(3, gray, black, black)
        surface_mapper = lambda group, material: surface  # noqa: E731
    model = ObjModel(text)
    if not model.faces:
        raise ValueError("the model has no faces")
    uv, pos, nrm, tng, groups, materials, tris = model.indexed()
    flip = uv.copy()
    flip[:, 1] = (F(1) - uv[:, 1]).astype(F)
    hack = name in ("aphroditegirl.obj", "smoothMonkey2.obj")
    prims = []
    prev_group, prev_material, start = "", "", 0

    def flush(t0, t1):
        corners = tris[t0:t1].reshape(-1)
        p, n, t = pos[corners], nrm[corners], tng[corners]
        if hack:
            p, n, t = _scale_hack(p, n, t)
        idx = np.arange(len(corners), dtype=np.int32).reshape(-1, 3)
        mesh = builder.mesh(p, idx, n, flip[corners], t)
        prims.append(builder.primitive(mesh, surface_mapper(prev_group, prev_material), position, rotation, scale))

    for k in range(len(tris)):
        g, m = groups[tris[k, 0]], materials[tris[k, 0]]
        if g != prev_group:
            if k > start:
                flush(start, k)
                start = k
            prev_group = g
        if m != prev_material:
            prev_material = m
    flush(start, len(tris))
    return prims
