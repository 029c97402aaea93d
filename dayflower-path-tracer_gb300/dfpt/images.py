"""Image decoding for ImageTexture.load (src/main/java/org/dayflower/pathtracer/scene/texture/
ImageTexture.java:470-479, 506-542): the reference reads a file with javax.imageio, draws it into a
TYPE_INT_RGB image (source-over onto black, so transparent texels become black) and keeps the
0x00RRGGBB ints in row-major order, top row first.

This module decodes the two formats the reference's textures use, from their published
specifications, with numpy only:
  * PNG (ISO/IEC 15948): colour types 0, 2, 3, 4, 6; bit depths 1-8 (palette, grey) and 8 (colour);
    tRNS transparency; no interlacing. Exact.
  * baseline JPEG (ITU-T T.81, sequential Huffman, 8-bit; SOF0/SOF1): any sampling factors, restart
    intervals, one or several scans of interleaved components. The inverse DCT is the separable
    float form of T.81 A.3.3, rounded to the nearest integer; colour conversion is JFIF's YCbCr to
    RGB; chroma is upsampled by replication. javax.imageio's decoder uses an integer IDCT and may
    differ by one level in some texels. Progressive JPEG (SOF2) is not decoded.

`load(path)` returns (width, height, uint32 array of 0x00RRGGBB).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"


def load(path):
    with open(path, "rb") as fh:
        data = fh.read()
    return decode(data)


def decode(data: bytes):
    if data[:8] == PNG_SIGNATURE:
        w, h, rgba = decode_png(data)
    elif data[:2] == b"\xff\xd8":
        w, h, rgba = decode_jpeg(data)
    else:
        raise ValueError("unknown image format (PNG and baseline JPEG are decoded)")
    return w, h, pack_rgb_over_black(rgba)


def pack_rgb_over_black(rgba: np.ndarray) -> np.ndarray:
    """RGBA8 (h, w, 4) drawn onto an opaque black TYPE_INT_RGB image, as 0x00RRGGBB ints.
    Alpha 255 copies the colour, alpha 0 leaves black; partial alpha scales the colour by a / 255
    (rounded)."""
    c = rgba[..., :3].astype(np.uint32)
    a = rgba[..., 3].astype(np.uint32)
    partial = (a != 255)
    if partial.any():
        c = np.where(partial[..., None], (c * a[..., None] + 127) // 255, c)
    return ((c[..., 0] << 16) | (c[..., 1] << 8) | c[..., 2]).reshape(-1).astype(np.uint32)


# PNG ---------------------------------------------------------------------------------------------

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw: bytes, height: int, stride: int, bpp: int) -> np.ndarray:
    """Reverses the per-scanline filters (PNG section 9): 0 none, 1 sub, 2 up, 3 average, 4 Paeth."""
    out = np.zeros((height, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(height):
        ftype = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 1:
            cur = line.copy()
            for k in range(bpp):  # running sum per byte lane
                cur[k::bpp] = np.cumsum(cur[k::bpp]) & 0xFF
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype == 3:
            cur = line.copy()
            for i in range(stride):
                left = cur[i - bpp] if i >= bpp else 0
                cur[i] = (cur[i] + ((left + prev[i]) >> 1)) & 0xFF
        elif ftype == 4:
            cur = line.copy()
            lst, pv = cur.tolist(), prev.tolist()
            for i in range(stride):
                a = lst[i - bpp] if i >= bpp else 0
                c = pv[i - bpp] if i >= bpp else 0
                lst[i] = (lst[i] + _paeth(a, pv[i], c)) & 0xFF
            cur = np.array(lst, np.int32)
        else:
            raise ValueError(f"PNG: bad filter type {ftype}")
        out[y] = cur
        prev = cur
    return out


def _unpack_bits(rows: np.ndarray, width: int, depth: int) -> np.ndarray:
    if depth == 8:
        return rows[:, :width]
    bits = np.unpackbits(rows, axis=1)
    per = bits.reshape(rows.shape[0], -1, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint8)
    vals = (per * weights).sum(axis=2).astype(np.uint8)
    return vals[:, :width]


def decode_png(data: bytes):
    if data[:8] != PNG_SIGNATURE:
        raise ValueError("not a PNG file")
    pos = 8
    idat = []
    palette = None
    trns = None
    hdr = None
    while pos + 8 <= len(data):
        length, ctype = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if ctype == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif ctype == b"tRNS":
            trns = body
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            break
    if hdr is None:
        raise ValueError("PNG: no IHDR")
    width, height, depth, color, _comp, _filt, interlace = hdr
    if interlace != 0:
        raise ValueError("PNG: interlaced images are not decoded")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}.get(color)
    if channels is None:
        raise ValueError(f"PNG: bad colour type {color}")
    if depth != 8 and not (color in (0, 3) and depth in (1, 2, 4)):
        raise ValueError(f"PNG: bit depth {depth} with colour type {color} is not decoded")
    bits_per_pixel = channels * depth
    stride = (width * bits_per_pixel + 7) // 8
    bpp = max(1, bits_per_pixel // 8)
    raw = zlib.decompress(b"".join(idat))
    if len(raw) < height * (stride + 1):
        raise ValueError("PNG: truncated image data")
    rows = _unfilter(raw, height, stride, bpp)
    rgba = np.full((height, width, 4), 255, np.uint8)
    if color == 3:
        if palette is None:
            raise ValueError("PNG: palette image without PLTE")
        idx = _unpack_bits(rows, width, depth)
        if idx.max(initial=0) >= len(palette):
            raise ValueError("PNG: palette index out of range")
        rgba[..., :3] = palette[idx]
        if trns is not None:
            alpha = np.full(len(palette), 255, np.uint8)
            t = np.frombuffer(trns, np.uint8)[:len(palette)]
            alpha[:len(t)] = t
            rgba[..., 3] = alpha[idx]
    elif color == 0:
        g = _unpack_bits(rows, width, depth).astype(np.uint16)
        scale = 255 // ((1 << depth) - 1)
        g8 = (g * scale).astype(np.uint8)
        rgba[..., 0] = rgba[..., 1] = rgba[..., 2] = g8
        if trns is not None and len(trns) >= 2:
            key = struct.unpack(">H", trns[:2])[0]
            rgba[..., 3] = np.where(g == key, 0, 255)
    else:
        px = rows[:, :width * channels].reshape(height, width, channels)
        if color == 2:
            rgba[..., :3] = px
            if trns is not None and len(trns) >= 6:
                key = np.array(struct.unpack(">HHH", trns[:6]))
                rgba[..., 3] = np.where((px == key).all(axis=2), 0, 255)
        elif color == 4:
            rgba[..., 0] = rgba[..., 1] = rgba[..., 2] = px[..., 0]
            rgba[..., 3] = px[..., 1]
        else:
            rgba[...] = px
    return width, height, rgba


# Baseline JPEG -----------------------------------------------------------------------------------

# Zig-zag scan order: position k of the coded sequence -> index in the 8 x 8 block (T.81 figure A.6).
def _zigzag():
    order = []
    for s in range(15):
        cells = [(i, s - i) for i in range(8) if 0 <= s - i < 8]
        if s % 2 == 0:
            cells.reverse()  # even diagonals run bottom-left to top-right
        order.extend(r * 8 + c for r, c in cells)
    return np.array(order)


ZIGZAG = _zigzag()


def _idct_matrix():
    # f(x) = sum_u C(u)/2 F(u) cos((2x+1) u pi / 16), C(0) = 1/sqrt(2)
    m = np.zeros((8, 8))
    for x in range(8):
        for u in range(8):
            cu = np.sqrt(0.5) if u == 0 else 1.0
            m[x, u] = 0.5 * cu * np.cos((2 * x + 1) * u * np.pi / 16.0)
    return m


IDCT = _idct_matrix()


class _Huffman:
    """Canonical Huffman table from BITS / HUFFVAL (T.81 annex C) as a 16-bit lookup."""

    def __init__(self, counts, symbols):
        self.lookup_sym = np.zeros(1 << 16, np.int32)
        self.lookup_len = np.zeros(1 << 16, np.int32)
        code = 0
        k = 0
        for length in range(1, 17):
            for _ in range(counts[length - 1]):
                lo = code << (16 - length)
                hi = (code + 1) << (16 - length)
                self.lookup_sym[lo:hi] = symbols[k]
                self.lookup_len[lo:hi] = length
                code += 1
                k += 1
            code <<= 1
        self.sym = self.lookup_sym.tolist()
        self.len = self.lookup_len.tolist()


class _Bits:
    """MSB-first bit reader over one entropy-coded segment (stuffed zero bytes removed)."""

    def __init__(self, seg: bytes):
        self.b = seg + b"\x00\x00\x00\x00"
        self.pos = 0  # bit position

    def peek16(self):
        p = self.pos >> 3
        b = self.b
        v = (b[p] << 16) | (b[p + 1] << 8) | b[p + 2]
        return (v >> (8 - (self.pos & 7))) & 0xFFFF

    def get(self, n):
        if n == 0:
            return 0
        p = self.pos >> 3
        b = self.b
        v = (b[p] << 24) | (b[p + 1] << 16) | (b[p + 2] << 8) | b[p + 3]
        r = (v >> (32 - (self.pos & 7) - n)) & ((1 << n) - 1)
        self.pos += n
        return r

    def decode(self, h: _Huffman):
        v = self.peek16()
        n = h.len[v]
        if n == 0:
            raise ValueError("JPEG: bad Huffman code")
        self.pos += n
        return h.sym[v]


def _extend(v, s):
    return v - (1 << s) + 1 if s and v < (1 << (s - 1)) else v


def _segments(data: bytes, start: int):
    """Splits the entropy-coded data after SOS at `start` into restart segments; returns them and
    the offset of the marker that ends the scan."""
    segs, cur = [], bytearray()
    i = start
    n = len(data)
    while i < n:
        c = data[i]
        if c != 0xFF:
            cur.append(c)
            i += 1
            continue
        m = data[i + 1] if i + 1 < n else 0xD9
        if m == 0x00:
            cur.append(0xFF)
            i += 2
        elif 0xD0 <= m <= 0xD7:
            segs.append(bytes(cur))
            cur = bytearray()
            i += 2
        elif m == 0xFF:
            i += 1  # fill byte
        else:
            break
    segs.append(bytes(cur))
    return segs, i


def decode_jpeg(data: bytes):
    if data[:2] != b"\xff\xd8":
        raise ValueError("not a JPEG file")
    qt = {}
    hts = {}
    restart = 0
    frame = None
    comps = []
    coef = None
    pos = 2
    while pos < len(data):
        if data[pos] != 0xFF:
            raise ValueError("JPEG: marker expected")
        m = data[pos + 1]
        if m == 0xFF:
            pos += 1
            continue
        if m == 0xD9:
            break
        if m in (0xD8,) or 0xD0 <= m <= 0xD7:
            pos += 2
            continue
        length = struct.unpack(">H", data[pos + 2:pos + 4])[0]
        body = data[pos + 4:pos + 2 + length]
        if m == 0xDB:  # DQT
            k = 0
            while k < len(body):
                pq, tq = body[k] >> 4, body[k] & 15
                if pq == 0:
                    vals = np.frombuffer(body, np.uint8, 64, k + 1).astype(np.int32)
                    k += 65
                else:
                    vals = np.frombuffer(body, ">u2", 64, k + 1).astype(np.int32)
                    k += 129
                q = np.zeros(64, np.int32)
                q[ZIGZAG] = vals
                qt[tq] = q
        elif m == 0xC4:  # DHT
            k = 0
            while k < len(body):
                tc, th = body[k] >> 4, body[k] & 15
                counts = list(body[k + 1:k + 17])
                total = sum(counts)
                syms = list(body[k + 17:k + 17 + total])
                hts[(tc, th)] = _Huffman(counts, syms)
                k += 17 + total
        elif m == 0xDD:  # DRI
            restart = struct.unpack(">H", body[:2])[0]
        elif m in (0xC0, 0xC1):
            precision, height, width, nc = struct.unpack(">BHHB", body[:6])
            if precision != 8:
                raise ValueError("JPEG: only 8-bit samples are decoded")
            comps = []
            for c in range(nc):
                cid, hv, tq = body[6 + 3 * c:9 + 3 * c]
                comps.append(dict(id=cid, h=hv >> 4, v=hv & 15, tq=tq))
            hmax = max(c["h"] for c in comps)
            vmax = max(c["v"] for c in comps)
            mcux = (width + 8 * hmax - 1) // (8 * hmax)
            mcuy = (height + 8 * vmax - 1) // (8 * vmax)
            for c in comps:
                c["bw"], c["bh"] = mcux * c["h"], mcuy * c["v"]
                c["coef"] = np.zeros((c["bh"], c["bw"], 64), np.int32)
            frame = (width, height, hmax, vmax, mcux, mcuy)
        elif 0xC2 <= m <= 0xCF and m not in (0xC4, 0xC8, 0xCC):
            raise ValueError("JPEG: progressive, lossless and arithmetic-coded files are not decoded")
        elif m == 0xDA:  # SOS
            if frame is None:
                raise ValueError("JPEG: scan before frame")
            ns = body[0]
            scomps = []
            for s in range(ns):
                cid, tdta = body[1 + 2 * s:3 + 2 * s]
                comp = next(c for c in comps if c["id"] == cid)
                scomps.append((comp, hts[(0, tdta >> 4)], hts[(1, tdta & 15)]))
            segs, end = _segments(data, pos + 2 + length)
            _decode_scan(frame, scomps, segs, restart)
            pos = end
            continue
        pos += 2 + length
    if frame is None:
        raise ValueError("JPEG: no frame")
    width, height, hmax, vmax, _, _ = frame
    planes = []
    for c in comps:
        blocks = c["coef"].astype(np.float64) * qt[c["tq"]][None, None, :]
        b = blocks.reshape(c["bh"], c["bw"], 8, 8)
        sp = np.einsum("xu,ijuv,yv->ijxy", IDCT, b, IDCT)  # rows: x over u, columns: y over v
        px = np.clip(np.floor(sp + 128.0 + 0.5), 0, 255)
        plane = px.transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)
        plane = np.repeat(np.repeat(plane, vmax // c["v"], axis=0), hmax // c["h"], axis=1)
        planes.append(plane[:height, :width])
    rgba = np.full((height, width, 4), 255, np.uint8)
    if len(planes) == 1:
        rgba[..., 0] = rgba[..., 1] = rgba[..., 2] = planes[0].astype(np.uint8)
    elif len(planes) == 3:
        y, cb, cr = planes[0], planes[1] - 128.0, planes[2] - 128.0
        r = y + 1.402 * cr
        g = y - 0.344136 * cb - 0.714136 * cr
        bl = y + 1.772 * cb
        for k, ch in enumerate((r, g, bl)):
            rgba[..., k] = np.clip(np.floor(ch + 0.5), 0, 255).astype(np.uint8)
    else:
        raise ValueError(f"JPEG: {len(planes)} components are not decoded")
    return width, height, rgba


def _decode_scan(frame, scomps, segs, restart):
    width, height, hmax, vmax, mcux, mcuy = frame
    if len(scomps) == 1:
        # Non-interleaved: one block per MCU, over the component's own block grid.
        comp, hdc, hac = scomps[0]
        bw = (int(np.ceil(width * comp["h"] / hmax)) + 7) // 8
        bh = (int(np.ceil(height * comp["v"] / vmax)) + 7) // 8
        units = [[(comp, hdc, hac, by, bx)] for by in range(bh) for bx in range(bw)]
    else:
        units = []
        for my in range(mcuy):
            for mx in range(mcux):
                u = []
                for comp, hdc, hac in scomps:
                    for v in range(comp["v"]):
                        for h in range(comp["h"]):
                            u.append((comp, hdc, hac, my * comp["v"] + v, mx * comp["h"] + h))
                units.append(u)
    per_seg = restart if restart else len(units)
    seg_i = 0
    for start in range(0, len(units), per_seg):
        if seg_i >= len(segs):
            raise ValueError("JPEG: missing restart segment")
        bits = _Bits(segs[seg_i])
        seg_i += 1
        pred = {id(c): 0 for c, _, _ in scomps}
        for u in units[start:start + per_seg]:
            for comp, hdc, hac, by, bx in u:
                blk = np.zeros(64, np.int32)
                s = bits.decode(hdc)
                diff = _extend(bits.get(s), s)
                pred[id(comp)] += diff
                blk[0] = pred[id(comp)]
                k = 1
                while k < 64:
                    rs = bits.decode(hac)
                    r, s = rs >> 4, rs & 15
                    if s == 0:
                        if r == 15:
                            k += 16
                            continue
                        break
                    k += r
                    if k > 63:
                        raise ValueError("JPEG: coefficient index out of range")
                    blk[ZIGZAG[k]] = _extend(bits.get(s), s)
                    k += 1
                comp["coef"][by, bx] = blk
