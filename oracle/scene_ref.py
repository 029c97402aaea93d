"""Pure-Python restatement of SceneCompiler + BoundingVolumeHierarchy. TEST INFRASTRUCTURE ONLY.

A second, independent restatement (float32 scalar arithmetic through numpy) of
  src/main/java/org/dayflower/pathtracer/scene/bvh/BoundingVolumeHierarchy.java:118-157, 805-986
  src/main/java/org/dayflower/pathtracer/scene/compiler/SceneCompiler.java:79-188, 888-995, 1034-1049
used by tests/ to check the C++ scene compiler of the product bit for bit on small scenes. It is
slow (pure Python loops) and meant for meshes of a few hundred triangles.
"""
from __future__ import annotations

import struct

import numpy as np

f32 = np.float32
FMAX = f32(3.4028234663852886e38)


def _key(*vals):
    out = []
    for v in vals:
        b = struct.unpack("<I", struct.pack("<f", float(f32(v))))[0]
        if (b & 0x7F800000) == 0x7F800000 and (b & 0x007FFFFF):
            b = 0x7FC00000
        out.append(b)
    return tuple(out)


class Distinct:
    def __init__(self):
        self.index, self.order = {}, []

    def add(self, k):
        if k not in self.index:
            self.index[k] = len(self.order)
            self.order.append(k)
        return self.index[k]


# ---- BVH --------------------------------------------------------------------------------------

class Node:
    def __init__(self, leaf, depth):
        self.leaf, self.depth = leaf, depth
        self.mx = self.my = self.mz = self.nx = self.ny = self.nz = f32(0)
        self.tris, self.left, self.right = [], None, None


def _build(items, depth, mx, my, mz, nx, ny, nz):
    size0 = len(items)
    if size0 < 4:
        n = Node(True, depth)
        n.tris = [it[6] for it in items]
        return n
    sx, sy, sz = f32(mx - nx), f32(my - ny), f32(mz - nz)
    min_cost = f32(f32(size0) * f32(f32(f32(sx * sy) + f32(sy * sz)) + f32(sz * sx)))
    best_split, best_axis = FMAX, -1
    for axis in range(3):
        start = (nx, ny, nz)[axis]
        stop = (mx, my, mz)[axis]
        if abs(f32(stop - start)) < f32(1.0e-4):
            continue
        step = f32(f32(stop - start) / f32(f32(1024.0) / f32(f32(depth) + f32(1.0))))
        split = f32(start + step)
        while split < f32(stop - step):
            lm = [-FMAX] * 3
            ln = [FMAX] * 3
            rm = [-FMAX] * 3
            rn = [FMAX] * 3
            cl = cr = 0
            for it in items:
                c = f32(f32(it[axis] + it[3 + axis]) * f32(0.5))
                if c < split:
                    for a in range(3):
                        lm[a] = max(lm[a], it[a])
                        ln[a] = min(ln[a], it[3 + a])
                    cl += 1
                else:
                    for a in range(3):
                        rm[a] = max(rm[a], it[a])
                        rn[a] = min(rn[a], it[3 + a])
                    cr += 1
            if cl > 1 and cr > 1:
                sl = [f32(lm[a] - ln[a]) for a in range(3)]
                sr = [f32(rm[a] - rn[a]) for a in range(3)]
                al = f32(f32(f32(sl[0] * sl[1]) + f32(sl[1] * sl[2])) + f32(sl[2] * sl[0]))
                ar = f32(f32(f32(sr[0] * sr[1]) + f32(sr[1] * sr[2])) + f32(sr[2] * sr[0]))
                cost = f32(f32(al * f32(cl)) + f32(ar * f32(cr)))
                if cost < min_cost:
                    min_cost, best_split, best_axis = cost, split, axis
            split = f32(split + step)
    if best_axis == -1:
        n = Node(True, depth)
        n.tris = [it[6] for it in items]
        return n
    left, right = [], []
    lm, ln, rm, rn = [-FMAX] * 3, [FMAX] * 3, [-FMAX] * 3, [FMAX] * 3
    for it in items:
        c = f32(f32(it[best_axis] + it[3 + best_axis]) * f32(0.5))
        if c < best_split:
            left.append(it)
            for a in range(3):
                lm[a] = max(lm[a], it[a]); ln[a] = min(ln[a], it[3 + a])
        else:
            right.append(it)
            for a in range(3):
                rm[a] = max(rm[a], it[a]); rn[a] = min(rn[a], it[3 + a])
    nl = _build(left, depth + 1, *lm, *ln)
    nl.mx, nl.my, nl.mz, nl.nx, nl.ny, nl.nz = *lm, *ln
    nr = _build(right, depth + 1, *rm, *rn)
    nr.mx, nr.my, nr.mz, nr.nx, nr.ny, nr.nz = *rm, *rn
    t = Node(False, depth)
    t.left, t.right = nl, nr
    return t


def build_bvh(tris):
    """tris: list of 3x(position) float32 triples. Returns the root Node."""
    items = []
    bm, bn = [-FMAX] * 3, [FMAX] * 3
    for i, (a, b, c) in enumerate(tris):
        it = [max(max(f32(a[k]), f32(b[k])), f32(c[k])) for k in range(3)] + \
             [min(min(f32(a[k]), f32(b[k])), f32(c[k])) for k in range(3)] + [i]
        items.append(it)
        for k in range(3):
            bm[k] = max(bm[k], it[k]); bn[k] = min(bn[k], it[3 + k])
    root = _build(items, 0, *bm, *bn)
    root.mx, root.my, root.mz, root.nx, root.ny, root.nz = *bm, *bn
    return root


def _size(n):
    return 5 + len(n.tris) if n.leaf else 5 + _size(n.left) + _size(n.right)


def _preorder(n, out):
    out.append(n)
    if not n.leaf:
        _preorder(n.left, out)
        _preorder(n.right, out)
    return out


def _bounds(n, d):
    d.add(_key(n.mx, n.my, n.mz))
    d.add(_key(n.nx, n.ny, n.nz))
    if not n.leaf:
        _bounds(n.left, d)
        _bounds(n.right, d)


def flatten(root, point_index, tri_offsets):
    """doCompileBoundingVolumeHierarchy: the literal 'search forward' definition of next/left."""
    nodes = _preorder(root, [])
    offs, j = [], 0
    for n in nodes:
        offs.append(j)
        j += 5 + (len(n.tris) if n.leaf else 0)
    out = []
    for i, n in enumerate(nodes):
        nxt = -1
        for k in range(i + 1, len(nodes)):
            if nodes[k].depth <= n.depth:
                nxt = offs[k]
                break
        mx = point_index[_key(n.mx, n.my, n.mz)] * 3
        mn = point_index[_key(n.nx, n.ny, n.nz)] * 3
        if n.leaf:
            out += [2, nxt, mn, mx, len(n.tris)] + [tri_offsets[t] for t in n.tris]
        else:
            left = -1
            for k in range(i + 1, len(nodes)):
                if nodes[k].depth == n.depth + 1:
                    left = offs[k]
                    break
            out += [1, nxt, mn, mx, left]
    return out


# ---- SceneCompiler ------------------------------------------------------------------------------

def compile_scene(desc):
    """desc: dict with 'textures' (records, blend children as indices), 'surfaces' (material, albedo,
    emission, normal, noise_amount, noise_scale), 'shapes' (('plane', a, b, c) | ('sphere', p, r) |
    ('mesh', vertices11, indices) | ('triangle', vertices11)), 'primitives' ((shape, surface, o2w16, w2o16)),
    'camera' (19 floats). Returns a dict of the 14 arrays."""
    shapes, prims, surfaces, textures = desc["shapes"], desc["primitives"], desc["surfaces"], desc["textures"]

    def tri_list(shape):
        v, idx = shape[1], shape[2] if shape[0] == "mesh" else [[0, 1, 2]]
        return [tuple(tuple(f32(x) for x in v[i]) for i in t) for t in idx]

    # Each mesh primitive builds its own BVH (the reference builds one per mesh, duplicates too).
    mesh_bvh = {}
    for si, _, _, _ in prims:
        if shapes[si][0] == "mesh" and si not in mesh_bvh:
            mesh_bvh[si] = build_bvh([tuple(vv[0:3] for vv in t) for t in tri_list(shapes[si])])
    # Textures: canonical value ids, then the collection order of doFindAllTextures.
    canon, dval = [], Distinct()
    for rec in textures:
        r = list(rec)
        if int(r[0]) == 1:
            r[2], r[3] = canon[int(r[2])], canon[int(r[3])]
        canon.append(dval.add(_key(*r)))
    dtex, tex_rep = Distinct(), []
    dsurf, surf_rep = Distinct(), []

    def skey(s):
        return (s[0], canon[s[1]], canon[s[2]], canon[s[3]]) + _key(s[4], s[5])

    def addt(ti):
        if canon[ti] not in dtex.index:
            tex_rep.append(ti)
        dtex.add(canon[ti])

    for si, sf, _, _ in prims:
        s = surfaces[sf]
        if skey(s) not in dsurf.index:
            surf_rep.append(sf)
        dsurf.add(skey(s))
        for ti in (s[1], s[2], s[3]):
            addt(ti)
        for ti in (s[1], s[2], s[3]):
            if int(textures[ti][0]) == 1:
                addt(int(textures[ti][2]))
                addt(int(textures[ti][3]))
    tex_off, o = {}, 0
    for ti in tex_rep:
        tex_off[canon[ti]] = o
        o += int(textures[ti][1])
    tex_arr = []
    for ti in tex_rep:
        r = list(textures[ti])
        if int(r[0]) == 1:
            r[2], r[3] = tex_off[canon[int(r[2])]], tex_off[canon[int(r[3])]]
        tex_arr += r
    surf_arr = []
    for sf in surf_rep:
        s = surfaces[sf]
        surf_arr += [s[0], tex_off[canon[s[1]]], tex_off[canon[s[2]]], tex_off[canon[s[3]]], s[4], s[5]]
    # Points, texture coordinates, vectors.
    p3, p2, v3 = Distinct(), Distinct(), Distinct()
    for si, _, _, _ in prims:
        if shapes[si][0] == "mesh":
            _bounds(mesh_bvh[si], p3)
    plane_normal = {}
    for si, _, _, _ in prims:
        s = shapes[si]
        if s[0] == "plane":
            for pnt in s[1:4]:
                p3.add(_key(*pnt))
        elif s[0] == "sphere":
            p3.add(_key(*s[1]))
        else:
            for t in tri_list(s):
                for vv in t:
                    p3.add(_key(*vv[0:3]))
    for si, _, _, _ in prims:
        s = shapes[si]
        if s[0] in ("mesh", "triangle"):
            for t in tri_list(s):
                for vv in t:
                    p2.add(_key(*vv[6:8]))
    for si, _, _, _ in prims:
        s = shapes[si]
        if s[0] == "plane":
            a, b, c = (np.asarray(x, np.float32) for x in s[1:4])
            ab, ac = b - a, c - a
            n = np.array([f32(f32(ab[1] * ac[2]) - f32(ab[2] * ac[1])), f32(f32(ab[2] * ac[0]) - f32(ab[0] * ac[2])),
                          f32(f32(ab[0] * ac[1]) - f32(ab[1] * ac[0]))], np.float32)
            ln = f32(np.sqrt(f32(f32(f32(n[0] * n[0]) + f32(n[1] * n[1])) + f32(n[2] * n[2]))))
            n = tuple(f32(x / ln) for x in n)
            plane_normal[si] = n
            v3.add(_key(*n))
        elif s[0] in ("mesh", "triangle"):
            for t in tri_list(s):
                for vv in t:
                    v3.add(_key(*vv[3:6]))
                for vv in t:
                    v3.add(_key(*vv[8:11]))

    def unpack(d):
        out = []
        for k in d.order:
            for w in k:
                out.append(struct.unpack("<f", struct.pack("<I", w))[0])
        return out or [0.0]

    arrays = {"point2fs": unpack(p2), "point3fs": unpack(p3), "vector3fs": unpack(v3)}
    # Shapes.
    dpl, dsp, dtr = Distinct(), Distinct(), Distinct()
    planes, spheres, tris = [], [], []
    shape_off, tri_offs = {}, {}
    for si, _, _, _ in prims:
        s = shapes[si]
        if s[0] == "plane":
            k = sum((_key(*x) for x in s[1:4]), ()) + _key(*plane_normal[si])
            new = k not in dpl.index
            shape_off[si] = dpl.add(k) * 4
            if new:
                planes += [p3.index[_key(*x)] * 3 for x in s[1:4]] + [v3.index[_key(*plane_normal[si])] * 3]
        elif s[0] == "sphere":
            k = _key(*s[1], s[2])
            new = k not in dsp.index
            shape_off[si] = dsp.add(k) * 2
            if new:
                spheres += [float(p3.index[_key(*s[1])] * 3), float(f32(s[2]))]
        else:
            offs = []
            for t in tri_list(s):
                k = sum((_key(*vv[6:8], *vv[0:3], *vv[3:6], *vv[8:11]) for vv in t), ())
                new = k not in dtr.index
                u = dtr.add(k)
                offs.append(u * 12)
                if new:
                    tris += [p3.index[_key(*vv[0:3])] * 3 for vv in t] + [v3.index[_key(*vv[3:6])] * 3 for vv in t] + \
                            [p2.index[_key(*vv[6:8])] * 2 for vv in t] + [v3.index[_key(*vv[8:11])] * 3 for vv in t]
            tri_offs.setdefault(si, offs)
            if s[0] == "triangle":
                shape_off[si] = offs[0]
    bvh, root_off = [], {}
    for si, _, _, _ in prims:
        if shapes[si][0] == "mesh" and si not in root_off:
            root_off[si] = len(bvh)
            bvh += flatten(mesh_bvh[si], p3.index, tri_offs[si])
    prim_arr, o2w, w2o = [], [], []
    type_id = {"plane": 1, "sphere": 2, "triangle": 4, "mesh": 5}
    for si, sf, m_o2w, m_w2o in prims:
        s = shapes[si]
        off = root_off[si] if s[0] == "mesh" else shape_off[si]
        prim_arr += [type_id[s[0]], off, dsurf.index[skey(surfaces[sf])] * 6]
        o2w += list(m_o2w)
        w2o += list(m_w2o)
    arrays.update({
        "planes": planes or [0], "spheres": spheres or [0.0], "terrains": [0.0], "triangles": tris or [0],
        "bounding_volume_hierarchies": bvh or [0], "textures": tex_arr or [0.0], "surfaces": surf_arr or [0.0],
        "primitives": prim_arr, "primitives_object_to_world": o2w, "primitives_world_to_object": w2o,
        "camera": list(desc["camera"]),
    })
    return arrays


# ---- Transform (Matrix44F translation * rotation * scale and its inverse, float32) --------------

def transform_matrices(position, quaternion, scale):
    px, py, pz = (f32(v) for v in position)
    qx, qy, qz, qw = (f32(v) for v in quaternion)
    sx, sy, sz = (f32(v) for v in scale)
    two, one = f32(2), f32(1)
    w = [f32(two * f32(f32(qx * qz) - f32(qw * qy))), f32(two * f32(f32(qy * qz) + f32(qw * qx))), f32(one - f32(two * f32(f32(qx * qx) + f32(qy * qy))))]
    v = [f32(two * f32(f32(qx * qy) + f32(qw * qz))), f32(one - f32(two * f32(f32(qx * qx) + f32(qz * qz)))), f32(two * f32(f32(qy * qz) - f32(qw * qx)))]
    u = [f32(one - f32(two * f32(f32(qy * qy) + f32(qz * qz)))), f32(two * f32(f32(qx * qy) - f32(qw * qz))), f32(two * f32(f32(qx * qz) + f32(qw * qy)))]
    T = [[one, 0, 0, px], [0, one, 0, py], [0, 0, one, pz], [0, 0, 0, one]]
    R = [u + [0], v + [0], w + [0], [0, 0, 0, one]]
    S = [[sx, 0, 0, 0], [0, sy, 0, 0], [0, 0, sz, 0], [0, 0, 0, one]]

    def mul(a, b):
        out = []
        for i in range(4):
            row = []
            for j in range(4):
                s = f32(f32(a[i][0]) * f32(b[0][j]))
                for k in range(1, 4):
                    s = f32(s + f32(f32(a[i][k]) * f32(b[k][j])))
                row.append(s)
            out.append(row)
        return out

    O = mul(mul(T, R), S)
    e = [f32(x) for row in O for x in row]
    e11, e12, e13, e14, e21, e22, e23, e24, e31, e32, e33, e34, e41, e42, e43, e44 = e

    def d(x, y, z, t):
        return f32(f32(x * y) - f32(z * t))
    a, b, c = d(e11, e22, e12, e21), d(e11, e23, e13, e21), d(e11, e24, e14, e21)
    dd, ee, f = d(e12, e23, e13, e22), d(e12, e24, e14, e22), d(e13, e24, e14, e23)
    g, h, i = d(e31, e42, e32, e41), d(e31, e43, e33, e41), d(e31, e44, e34, e41)
    j, k, l = d(e32, e43, e33, e42), d(e32, e44, e34, e42), d(e33, e44, e34, e43)
    det = f32(f32(f32(f32(f32(f32(a * l) - f32(b * k)) + f32(c * j)) + f32(dd * i)) - f32(ee * h)) + f32(f * g))
    r = f32(f32(1) / det)

    def t3(x1, y1, x2, y2, x3, y3, sign):
        v = f32(f32(f32(sign[0] * f32(x1 * y1)) + f32(sign[1] * f32(x2 * y2))) + f32(sign[2] * f32(x3 * y3)))
        return f32(v * r)
    P, N = f32(1), f32(-1)
    inv = [
        t3(e22, l, e23, k, e24, j, (P, N, P)), t3(e12, l, e13, k, e14, j, (N, P, N)), t3(e42, f, e43, ee, e44, dd, (P, N, P)), t3(e32, f, e33, ee, e34, dd, (N, P, N)),
        t3(e21, l, e23, i, e24, h, (N, P, N)), t3(e11, l, e13, i, e14, h, (P, N, P)), t3(e41, f, e43, c, e44, b, (N, P, N)), t3(e31, f, e33, c, e34, b, (P, N, P)),
        t3(e21, k, e22, i, e24, g, (P, N, P)), t3(e11, k, e12, i, e14, g, (N, P, N)), t3(e41, ee, e42, c, e44, a, (P, N, P)), t3(e31, ee, e32, c, e34, a, (N, P, N)),
        t3(e21, j, e22, h, e23, g, (N, P, N)), t3(e11, j, e12, h, e13, g, (P, N, P)), t3(e41, dd, e42, b, e43, a, (N, P, N)), t3(e31, dd, e32, b, e33, a, (P, N, P)),
    ]
    return [float(x) for x in e], [float(x) for x in inv]
