"""Test helpers: a PNG writer and a minimal baseline JPEG encoder (to check dfpt.images against
files with known content), and a synthetic resource directory with the reference's file names (so
the named-scene builders run where the reference's resources are absent)."""
import struct
import zlib

import numpy as np

from dfpt import images

# PNG ---------------------------------------------------------------------------------------------

def chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def filter_row(kind, row, prev, bpp):
    row = row.astype(np.int32)
    prev = prev.astype(np.int32)
    out = np.zeros_like(row)
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        if kind == 0:
            pred = 0
        elif kind == 1:
            pred = a
        elif kind == 2:
            pred = b
        elif kind == 3:
            pred = (a + b) >> 1
        else:
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
        out[i] = (row[i] - pred) & 0xFF
    return out.astype(np.uint8)


def png(rows, width, height, depth, color, palette=None, trns=None):
    bpp = max(1, {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[color] * depth // 8)
    raw = bytearray()
    prev = np.zeros(rows.shape[1], np.uint8)
    for y in range(height):
        kind = y % 5
        raw.append(kind)
        raw += filter_row(kind, rows[y], prev, bpp).tobytes()
        prev = rows[y]
    out = images.PNG_SIGNATURE + chunk(b"IHDR", struct.pack(">IIBBBBB", width, height, depth, color, 0, 0, 0))
    if palette is not None:
        out += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        out += chunk(b"tRNS", trns)
    return out + chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b"")


# Baseline JPEG -----------------------------------------------------------------------------------

def _huff_table(symbols):
    """Every symbol gets an 8-bit code (at most 255 symbols, so the all-ones code stays unused)."""
    symbols = sorted(set(symbols))
    assert len(symbols) <= 255
    counts = [0] * 16
    counts[7] = len(symbols)
    codes = {s: (k, 8) for k, s in enumerate(symbols)}
    return counts, symbols, codes


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, length):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)  # byte stuffing
                self.acc = 0
                self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)  # pad with ones
        data = bytes(self.out)
        self.out = bytearray()
        return data


def _category(v):
    v = abs(int(v))
    return v.bit_length()


def _bits_of(v, s):
    return v if v >= 0 else v + (1 << s) - 1


def encode_jpeg(rgb, sub=1, restart=0, q=1):
    h, w, _ = rgb.shape
    x = rgb.astype(np.float64)
    y = 0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]
    cb = -0.168736 * x[..., 0] - 0.331264 * x[..., 1] + 0.5 * x[..., 2] + 128.0
    cr = 0.5 * x[..., 0] - 0.418688 * x[..., 1] - 0.081312 * x[..., 2] + 128.0
    mcu = 8 * sub
    mx, my = (w + mcu - 1) // mcu, (h + mcu - 1) // mcu

    def pad(p, hh, ww):
        return np.pad(p, ((0, hh - p.shape[0]), (0, ww - p.shape[1])), mode="edge")

    planes = [pad(y, my * mcu, mx * mcu)]
    for c in (cb, cr):
        c = pad(c, my * mcu, mx * mcu)
        if sub == 2:
            c = c.reshape(my * 8, 2, mx * 8, 2).mean(axis=(1, 3))
        planes.append(c)
    samp = [(sub, sub), (1, 1), (1, 1)]
    quant = np.full(64, q, np.int32)

    def blocks(plane):
        bh, bw = plane.shape[0] // 8, plane.shape[1] // 8
        b = plane.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3) - 128.0
        coef = np.einsum("ux,ijxy,yv->ijuv", images.IDCT.T, b, images.IDCT)
        return np.round(coef.reshape(bh, bw, 64) / quant).astype(np.int64)

    coefs = [blocks(p) for p in planes]
    units = []
    for j in range(my):
        for i in range(mx):
            u = []
            for c, (hs, vs) in enumerate(samp):
                for v in range(vs):
                    for hh in range(hs):
                        u.append((c, coefs[c][j * vs + v, i * hs + hh]))
            units.append(u)
    # Symbols, then tables.
    dc_syms, ac_syms = set(), set()
    pred = [0, 0, 0]
    for k, u in enumerate(units):
        if restart and k % restart == 0:
            pred = [0, 0, 0]
        for c, blk in u:
            z = blk[images.ZIGZAG]
            dc_syms.add(_category(z[0] - pred[c]))
            pred[c] = z[0]
            run = 0
            last = max([i for i in range(1, 64) if z[i] != 0], default=0)
            for i in range(1, last + 1):
                if z[i] == 0:
                    run += 1
                    if run == 16:
                        ac_syms.add(0xF0)
                        run = 0
                    continue
                ac_syms.add((run << 4) | _category(z[i]))
                run = 0
            if last < 63:
                ac_syms.add(0x00)
    dc = _huff_table(dc_syms)
    ac = _huff_table(ac_syms)
    bw = _BitWriter()
    segments = []
    pred = [0, 0, 0]
    for k, u in enumerate(units):
        if restart and k and k % restart == 0:
            segments.append(bw.flush())
            pred = [0, 0, 0]
        for c, blk in u:
            z = blk[images.ZIGZAG]
            d = int(z[0] - pred[c])
            pred[c] = int(z[0])
            s = _category(d)
            bw.put(*dc[2][s])
            bw.put(_bits_of(d, s), s)
            run = 0
            last = max([i for i in range(1, 64) if z[i] != 0], default=0)
            for i in range(1, last + 1):
                if z[i] == 0:
                    run += 1
                    if run == 16:
                        bw.put(*ac[2][0xF0])
                        run = 0
                    continue
                s = _category(z[i])
                bw.put(*ac[2][(run << 4) | s])
                bw.put(_bits_of(int(z[i]), s), s)
                run = 0
            if last < 63:
                bw.put(*ac[2][0x00])
    segments.append(bw.flush())
    scan = bytearray()
    for k, seg in enumerate(segments):
        if k:
            scan += bytes([0xFF, 0xD0 + (k - 1) % 8])
        scan += seg

    def seg(marker, body):
        return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body

    out = b"\xff\xd8"
    out += seg(0xDB, bytes([0]) + bytes(quant[images.ZIGZAG].astype(np.uint8)))
    sof = struct.pack(">BHHB", 8, h, w, 3)
    for c, (hs, vs) in enumerate(samp):
        sof += bytes([c + 1, (hs << 4) | vs, 0])
    out += seg(0xC0, sof)
    for tc, (counts, syms, _) in ((0, dc), (1, ac)):
        out += seg(0xC4, bytes([tc << 4]) + bytes(counts) + bytes(syms))
    if restart:
        out += seg(0xDD, struct.pack(">H", restart))
    sos = bytes([3]) + b"".join(bytes([c + 1, 0x00]) for c in range(3)) + bytes([0, 63, 0])
    out += seg(0xDA, sos) + bytes(scan) + b"\xff\xd9"
    return out


def smooth_image(h, w, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.zeros((h, w, 3))
    for c in range(3):
        fx, fy, ph = rng.uniform(0.01, 0.08), rng.uniform(0.01, 0.08), rng.uniform(0, 6)
        img[..., c] = 128 + 100 * np.sin(fx * xx + ph) * np.cos(fy * yy) + 0.2 * xx - 0.1 * yy
    return np.clip(np.round(img), 0, 255).astype(np.uint8)




def sphere_obj(subdivisions=2, radius=0.5, groups=(("g0", "m0"),), normals=False, center=(0.0, 0.0, 0.0)):
    """OBJ text of a geodesic sphere: `v`, spherical `vt`, optional `vn`, faces split evenly over
    the (group, material) pairs."""
    from dfpt.synthetic import geodesic_sphere

    pos, idx = geodesic_sphere(subdivisions)[:2]
    pos = np.asarray(pos, np.float64)
    pos = pos / np.linalg.norm(pos, axis=1, keepdims=True)
    lines = [f"v {c[0] + radius * x:.6f} {c[1] + radius * y:.6f} {c[2] + radius * z:.6f}" for (x, y, z), c in
             zip(pos, [center] * len(pos))]
    u = 0.5 + np.arctan2(pos[:, 2], pos[:, 0]) / (2 * np.pi)
    v = 0.5 - np.arcsin(np.clip(pos[:, 1], -1, 1)) / np.pi
    lines += [f"vt {a:.6f} {b:.6f}" for a, b in zip(u, v)]
    if normals:
        lines += [f"vn {x:.6f} {y:.6f} {z:.6f}" for x, y, z in pos]
    per = (len(idx) + len(groups) - 1) // len(groups)
    for k, (a, b, c) in enumerate(idx):
        if k % per == 0:
            g, m = groups[k // per]
            lines += [f"g {g}", f"usemtl {m}"]
        if normals:
            lines.append(f"f {a + 1}/{a + 1}/{a + 1} {b + 1}/{b + 1}/{b + 1} {c + 1}/{c + 1}/{c + 1}")
        else:
            lines.append(f"f {a + 1}/{a + 1} {b + 1}/{b + 1} {c + 1}/{c + 1}")
    return "\n".join(lines) + "\n"


def write_resources(root):
    """A resource directory (model/, texture/) under the reference's file names with synthetic
    content: a 64 x 64 palette PNG with a transparent entry for Texture_2.png, a smooth 64 x 64
    normal-map JPEG for bricks2_normal.jpg, and geodesic spheres for the OBJ models."""
    import os

    rng = np.random.default_rng(7)
    os.makedirs(os.path.join(root, "model"), exist_ok=True)
    os.makedirs(os.path.join(root, "texture"), exist_ok=True)
    idx = rng.integers(0, 16, (64, 64)).astype(np.uint8)
    palette = rng.integers(0, 256, (16, 3))
    with open(os.path.join(root, "texture", "Texture_2.png"), "wb") as f:
        f.write(png(idx, 64, 64, 8, 3, palette=palette, trns=bytes([0])))
    yy, xx = np.mgrid[0:64, 0:64] / 64.0
    nx, ny = 0.3 * np.sin(6.0 * xx), 0.3 * np.cos(5.0 * yy)
    nz = np.sqrt(1.0 - nx ** 2 - ny ** 2)
    nmap = np.clip(np.round((np.stack([nx, ny, nz], -1) + 1.0) * 127.5), 0, 255).astype(np.uint8)
    with open(os.path.join(root, "texture", "bricks2_normal.jpg"), "wb") as f:
        f.write(encode_jpeg(nmap, q=2))
    models = {
        "smoothMonkey2.obj": sphere_obj(3, 0.5),
        "aphroditegirl.obj": sphere_obj(3, 0.4, groups=(("body", "01___Default"), ("dress", "02___Default"),
                                                       ("hair", "no_such_material"))),
        "Wine_Glass.OBJ": sphere_obj(2, 0.4, normals=True),
    }
    for name, text in models.items():
        with open(os.path.join(root, "model", name), "w") as f:
            f.write(text)
    return root
