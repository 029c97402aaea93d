"""Generates the golden fixtures in tests/golden/ (run from the repository root).

    python tests/golden/make_golden.py

Each known-answer set is computed here by a pure-Python restatement written independently of the
C++ oracle and the CUDA core, from the reference's formulas:
  philox.json    Philox4x32-10 known-answer vectors published with Random123 (Salmon et al.)
  lcg.json       AbstractKernel.doNext/nextFloat (AbstractKernel.java:438-440, 1101-1110), integer LCG
  noise.json     simplexNoiseXYZ / simplexFractionalBrownianMotionXYZ (AbstractKernel.java:695-716, 812-900)
  sky.json       Sky.set + doCalculateColorForSky (Sky.java:295-333, GPURendererKernel.java:2127-2236), FP64
  tonemap.json   tone maps, sRGB redo-gamma, BGRA8 (AbstractImageKernel.java:428-534, 702-774)
  intersect.json analytic ray/sphere, ray/plane and ray/triangle answers
  render_*.npz   small compiled scenes with oracle renders (FP64 path tracer, strict-FP32 ray caster)
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "dayflower-path-tracer_gb300"))
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent
f32 = np.float32

PERM_SRC = None


def perm():
    global PERM_SRC
    if PERM_SRC is None:
        from dfpt.noise_tables import PERMUTATION

        PERM_SRC = PERMUTATION + PERMUTATION
    return PERM_SRC


GRAD3 = [(1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0), (1, 0, 1), (-1, 0, 1), (1, 0, -1), (-1, 0, -1), (0, 1, 1),
         (0, -1, 1), (0, 1, -1), (0, -1, -1)]


def fast_floor(v):
    i = int(v)
    return i - 1 if v < f32(i) else i


def simplex3(x, y, z):
    P = perm()
    x, y, z = f32(x), f32(y), f32(z)
    F3, G3 = f32(1.0 / 3.0), f32(1.0 / 6.0)
    s = f32(f32(f32(x + y) + z) * F3)
    i, j, k = fast_floor(f32(x + s)), fast_floor(f32(y + s)), fast_floor(f32(z + s))
    t = f32(f32(i + j + k) * G3)
    x0, y0, z0 = f32(x - f32(f32(i) - t)), f32(y - f32(f32(j) - t)), f32(z - f32(f32(k) - t))
    if x0 >= y0:
        if y0 >= z0:
            o1, o2 = (1, 0, 0), (1, 1, 0)
        elif x0 >= z0:
            o1, o2 = (1, 0, 0), (1, 0, 1)
        else:
            o1, o2 = (0, 0, 1), (1, 0, 1)
    else:
        if y0 < z0:
            o1, o2 = (0, 0, 1), (0, 1, 1)
        elif x0 < z0:
            o1, o2 = (0, 1, 0), (0, 1, 1)
        else:
            o1, o2 = (0, 1, 0), (1, 1, 0)
    corners = [(x0, y0, z0, (0, 0, 0)),
               (f32(f32(x0 - o1[0]) + G3), f32(f32(y0 - o1[1]) + G3), f32(f32(z0 - o1[2]) + G3), o1),
               (f32(f32(x0 - o2[0]) + f32(2 * G3)), f32(f32(y0 - o2[1]) + f32(2 * G3)), f32(f32(z0 - o2[2]) + f32(2 * G3)), o2),
               (f32(f32(x0 - 1) + f32(3 * G3)), f32(f32(y0 - 1) + f32(3 * G3)), f32(f32(z0 - 1) + f32(3 * G3)), (1, 1, 1))]
    ii, jj, kk = i & 255, j & 255, k & 255
    n = f32(0)
    total = []
    for cx, cy, cz, o in corners:
        gi = P[ii + o[0] + P[jj + o[1] + P[kk + o[2]]]] % 12
        tt = f32(f32(f32(f32(0.6) - f32(cx * cx)) - f32(cy * cy)) - f32(cz * cz))
        g = GRAD3[gi]
        dot = f32(f32(f32(f32(g[0]) * cx) + f32(f32(g[1]) * cy)) + f32(f32(g[2]) * cz))
        total.append(f32(0) if tt < 0 else f32(f32(f32(tt * tt) * f32(tt * tt)) * dot))
    n = f32(f32(f32(total[0] + total[1]) + total[2]) + total[3])
    return float(f32(f32(32) * n))


def fbm3(freq, gain, mn, mx, octaves, x, y, z):
    amp, maxamp, fr, noise = f32(1), f32(0), f32(freq), f32(0)
    for _ in range(octaves):
        noise = f32(noise + f32(f32(simplex3(f32(x * fr), f32(y * fr), f32(z * fr))) * amp))
        maxamp = f32(maxamp + amp)
        amp = f32(amp * f32(gain))
        fr = f32(fr * f32(2))
    noise = f32(noise / maxamp)
    return float(f32(f32(f32(noise * f32(f32(mx) - f32(mn))) / f32(2)) + f32(f32(f32(mx) + f32(mn)) / f32(2))))


def lcg_floats(seed, count):
    out, s = [], seed
    for _ in range(count):
        s = (s * 0x5DEECE66D + 0xB) & ((1 << 48) - 1)
        out.append(float(f32(f32(s >> 24) * f32(1.0 / (1 << 24)))))
    return out


def sky_rgb(sun_dir_world, turbidity, direction):
    """Sky.set then doCalculateColorForSky, in FP64 except where the reference narrows to float."""
    v = np.asarray(sun_dir_world, np.float32)
    ln = f32(math.sqrt(float(f32(f32(f32(v[0] * v[0]) + f32(v[1] * v[1])) + f32(v[2] * v[2])))))
    dw = [f32(c / ln) for c in v]
    sd = [dw[0], dw[2], dw[1]]  # the sky basis u = X, v = Z, w = Y
    sl = f32(math.sqrt(float(f32(f32(f32(sd[0] * sd[0]) + f32(sd[1] * sd[1])) + f32(sd[2] * sd[2])))))
    sd = [f32(c / sl) for c in sd]
    theta = float(f32(math.acos(min(max(float(sd[2]), -1.0), 1.0))))
    T = float(f32(turbidity))
    chi = (4.0 / 9.0 - T / 120.0) * (float(f32(math.pi)) - 2.0 * theta)
    zl = ((4.0453 * T - 4.9710) * math.tan(chi) - 0.2155 * T + 2.4192) * 1000.0
    th2, th3 = theta * theta, theta ** 3
    zx = (0.00165 * th3 - 0.00374 * th2 + 0.00208 * theta) * T * T + (-0.02902 * th3 + 0.06377 * th2 - 0.03202 * theta + 0.00394) * T + (0.11693 * th3 - 0.21196 * th2 + 0.06052 * theta + 0.25885)
    zy = (0.00275 * th3 - 0.00610 * th2 + 0.00316 * theta) * T * T + (-0.04212 * th3 + 0.08970 * th2 - 0.04153 * theta + 0.00515) * T + (0.15346 * th3 - 0.26756 * th2 + 0.06669 * theta + 0.26688)
    L = [0.17872 * T - 1.46303, -0.35540 * T + 0.42749, -0.02266 * T + 5.32505, 0.12064 * T - 2.57705, -0.06696 * T + 0.37027]
    X = [-0.01925 * T - 0.25922, -0.06651 * T + 0.00081, -0.00041 * T + 0.21247, -0.06409 * T - 0.89887, -0.00325 * T + 0.04517]
    Y = [-0.01669 * T - 0.26078, -0.09495 * T + 0.00921, -0.00792 * T + 0.21023, -0.04405 * T - 1.65369, -0.01092 * T + 0.05291]
    d = [float(c) for c in direction]
    d0 = [d[0], d[2], d[1]]
    if d0[2] < 0:
        return [0.01, 0.01, 0.01]
    d0[2] = max(d0[2], 0.001)
    ln = math.sqrt(sum(c * c for c in d0))
    d1 = [c / ln for c in d0]
    dp = sum(d1[i] * float(sd[i]) for i in range(3))
    th1 = math.acos(max(min(d1[2], 1.0), -1.0))
    c0, c1 = math.cos(theta), math.cos(th1)
    c1r = 1.0 / (c1 + 0.01)
    gamma = math.acos(max(min(dp, 1.0), -1.0))
    cg = math.cos(gamma)
    rel = zl * ((1 + L[0] * math.exp(L[1] * c1r)) * (1 + L[2] * math.exp(L[3] * gamma) + L[4] * cg * cg)) / \
        ((1 + L[0] * math.exp(L[1])) * (1 + L[2] * math.exp(L[3] * theta) + L[4] * c0 * c0)) * 1e-4
    x = zx * ((1 + X[0] * math.exp(X[1] * c1r)) * (1 + X[2] * math.exp(X[3] * gamma) + X[4] * cg * cg)) / \
        ((1 + X[0] * math.exp(X[1])) * (1 + X[2] * math.exp(X[3] * th1) + X[4] * c0 * c0))
    y = zy * ((1 + Y[0] * math.exp(Y[1] * c1r)) * (1 + Y[2] * math.exp(Y[3] * gamma) + Y[4] * cg * cg)) / \
        ((1 + Y[0] * math.exp(Y[1])) * (1 + Y[2] * math.exp(Y[3] * th1) + Y[4] * c0 * c0))
    k0 = 1.0 / (0.0241 + 0.2562 * x - 0.7341 * y)
    k1 = (-1.3515 - 1.7703 * x + 5.9114 * y) * k0
    k2 = (0.03 - 31.4424 * x + 30.0717 * y) * k0
    cx = 10246.121 + k1 * 187.75537 + k2 * 213.14803
    cy = 10676.695 + k1 * 192.59653 + k2 * 76.29494
    cz = 12372.504 + k1 * 3482.8765 + k2 * -235.71611
    R, G, B = cx * rel / cy, rel, cz * rel / cy
    r = 3.2410042 * R - 1.5373994 * G - 0.49861607 * B
    g = -0.9692241 * R + 1.8759298 * G + 0.041554242 * B
    b = 0.05563942 * R - 0.20401107 * G + 1.0571486 * B
    w = max(0.0, -min(0.0, min(r, min(g, b))))
    return [r + w, g + w, b + w]


def tonemap(kind, exposure, rgb):
    """Tone map + RGBColorSpace.SRGB redo gamma + clamp to bytes, float32 arithmetic."""
    e = f32(exposure)
    out = []
    bp, gm = f32(0.00304), f32(2.4)
    pe = f32(math.pow(float(bp), float(f32(f32(1) / gm) - f32(1))))
    slope = f32(f32(1) / f32(f32(f32(gm / pe) - f32(gm * bp)) + bp))
    match = f32(f32(gm * slope) / pe)
    seg = f32(f32(match * f32(math.pow(float(bp), float(f32(f32(1) / gm))))) - f32(slope * bp))
    for v in (f32(c) for c in rgb):
        if kind == 2:
            m = f32(v * e)
            v = f32(m / f32(f32(1) + m))
        elif kind == 3:
            v = f32(f32(1) - f32(math.exp(float(f32(-v * e)))))
        elif kind == 4:
            lw = f32(f32(1) / f32(16))
            m = f32(v * e)
            v = f32(f32(m * f32(f32(1) + f32(m * lw))) / f32(f32(1) + m))
        elif kind == 1:
            m = max(f32(v * e), f32(-3.4028234663852886e38))
            q = f32(f32(m * f32(f32(f32(2.51) * m) + f32(0.03))) / f32(f32(m * f32(f32(f32(2.43) * m) + f32(0.59))) + f32(0.14)))
            v = f32(0) if q < 0 else f32(1) if q > 1 else q
        if v <= 0:
            v = f32(0)
        elif v >= 1:
            v = f32(1)
        elif v <= bp:
            v = f32(v * slope)
        else:
            v = f32(f32(match * f32(math.pow(float(v), float(f32(f32(1) / gm))))) - seg)
        out.append(int(max(min(float(f32(f32(v * f32(255)) + f32(0.5))), 255.0), 0.0)))
    return [out[2], out[1], out[0], 255]


def main():
    (OUT / "philox.json").write_text(json.dumps({"source": "Random123 known-answer vectors for philox4x32_10", "cases": [
        {"counter": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]},
        {"counter": [0xffffffff] * 4, "key": [0xffffffff] * 2, "out": [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]},
        {"counter": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], "key": [0xa4093822, 0x299f31d0],
         "out": [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]}]}, indent=1))
    states = [0, 1, 42, 0x123456789ABC, (1 << 48) - 1]
    (OUT / "lcg.json").write_text(json.dumps({"cases": [{"state": s, "floats": lcg_floats(s, 8)} for s in states]}, indent=1))
    rng = np.random.default_rng(11)
    pts = rng.uniform(-20, 20, (24, 3)).astype(np.float32)
    (OUT / "noise.json").write_text(json.dumps({
        "simplex3": [[float(p[0]), float(p[1]), float(p[2]), simplex3(*p)] for p in pts],
        "fbm3": [[float(p[0]), float(p[1]), float(p[2]), fbm3(0.5, 0.5, -0.26, 0.26, 16, *p)] for p in pts[:8]]}, indent=1))
    dirs = [(0, 1, 0), (0.5, 0.70710677, 0.5), (1, 0.1, 0), (0, 0.3, -1), (-0.3, 0.9, 0.2), (0.2, 0.0005, 0.9), (0, -0.5, 1)]
    (OUT / "sky.json").write_text(json.dumps({"sun_direction_world": [0.5, 0.70710677, 0.5], "turbidity": 2.0, "cases": [
        {"direction": list(d), "rgb": sky_rgb((0.5, 0.70710677, 0.5), 2.0, d)} for d in dirs]}, indent=1))
    vals = [[0.0, 0.0, 0.0], [0.001, 0.002, 0.003], [0.18, 0.5, 0.9], [1.0, 2.0, 4.0], [25.0, 0.0004, 7.5]]
    (OUT / "tonemap.json").write_text(json.dumps({"cases": [{"kind": k, "exposure": e, "rgb": v, "bgra": tonemap(k, e, v)}
                                                           for k in (1, 2, 3, 4) for e in (1.0, 0.5) for v in vals]}, indent=1))
    (OUT / "intersect.json").write_text(json.dumps({"note": "analytic answers; sphere at origin radius 2, plane y=0, triangle (0,0,0),(1,0,0),(0,1,0)", "cases": [
        {"shape": "sphere", "ray": [0, 0, -10, 0, 0, 1], "t": 8.0, "normal": [0, 0, -1]},
        {"shape": "sphere", "ray": [0, 0, 0, 1, 0, 0], "t": 2.0, "normal": [1, 0, 0]},
        {"shape": "sphere", "ray": [0, 5, -10, 0, 0, 1], "t": None},
        {"shape": "plane", "ray": [3, 4, 5, 0, -1, 0], "t": 4.0, "normal": [0, 1, 0]},
        {"shape": "plane", "ray": [3, 4, 5, 1, 0, 0], "t": None},
        {"shape": "triangle", "ray": [0.25, 0.25, -3, 0, 0, 1], "t": 3.0, "normal": [0, 0, 1]},
        {"shape": "triangle", "ray": [0.75, 0.75, -3, 0, 0, 1], "t": None}]}, indent=1))
    make_renders()


def make_renders():
    from dfpt import synthetic
    from dfpt.kernel import default_params
    from oracle import oracle

    for name, (scene, sky, params, _) in {"spheres": synthetic.sphere_scene(0, 32, 24),
                                          "meshes": synthetic.small_mesh_scene(width=32, height=24)}.items():
        w, h = 32, 24
        p = default_params()
        for k, v in params.items():
            setattr(p, k, v)
        pt = oracle.render(scene, sky, p, w, h, passes=16, precision=64)
        p.renderer_type = 3
        rc = oracle.render(scene, sky, p, w, h, passes=1, precision=32, hits=True, want_bgra=True)
        np.savez_compressed(OUT / f"render_{name}.npz", width=w, height=h, params=json.dumps(params),
                            sky=json.dumps(sky.as_dict()), pt_film=pt["film"], pt_passes=16,
                            rc_hit_prim=rc["hit_prim"], rc_hit_off=rc["hit_off"], rc_hit_dist=rc["hit_dist"],
                            rc_hit_normal=rc["hit_normal"], rc_bgra=rc["bgra"], **{f"scene_{k}": v for k, v in scene.arrays().items()})


if __name__ == "__main__":
    main()
