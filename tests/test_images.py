"""CPU: the image decoders behind ImageTexture.load (dfpt.images).

PNG decoding is exact: images written here with every scanline filter, colour type and small bit
depth decode to the pixels they were made from. Baseline JPEG is checked end to end against a
minimal encoder written here (forward DCT, quantisation, canonical Huffman codes, byte stuffing,
restart markers): with unit quantisation the decoded pixels stay within a few levels of the source
(4:4:4) and within a wider bound with 2 x 2 chroma subsampling. The reference's own texture files,
when present, decode to their stated sizes.
"""
from pathlib import Path

import numpy as np
import pytest

from _imaging import encode_jpeg, png, smooth_image
from conftest import reference_resources
from dfpt import images

_RES = reference_resources()
TEX = _RES / "texture" if _RES else Path("missing-reference-resources")


def _unpack(v):
    return (v >> 16) & 255, (v >> 8) & 255, v & 255


def test_png_rgb_and_rgba_all_filters():
    rng = np.random.default_rng(1)
    w, h = 37, 11
    rgb = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    ww, hh, data = images.decode(png(rgb.reshape(h, -1), w, h, 8, 2))
    assert (ww, hh) == (w, h)
    r, g, b = _unpack(data.reshape(h, w))
    assert np.array_equal(np.stack([r, g, b], -1), rgb)
    # RGBA: opaque texels keep their colour, transparent ones turn black (drawn onto black).
    a = np.where(rng.random((h, w)) < 0.3, 0, 255).astype(np.uint8)
    rgba = np.concatenate([rgb, a[..., None]], -1)
    _, _, data = images.decode(png(rgba.reshape(h, -1), w, h, 8, 6))
    r, g, b = _unpack(data.reshape(h, w))
    expect = np.where(a[..., None] == 255, rgb, 0)
    assert np.array_equal(np.stack([r, g, b], -1), expect)


@pytest.mark.parametrize("depth", [1, 2, 4, 8])
def test_png_palette_and_grey_bit_depths(depth):
    rng = np.random.default_rng(depth)
    w, h = 29, 7
    n = 1 << depth
    idx = rng.integers(0, n, (h, w))
    per_byte = 8 // depth
    packed = np.zeros((h, (w + per_byte - 1) // per_byte), np.uint8)
    for x in range(w):
        packed[:, x // per_byte] |= (idx[:, x] << (8 - depth * (x % per_byte + 1))).astype(np.uint8)
    palette = rng.integers(0, 256, (n, 3))
    trns = bytes([0]) if depth == 8 else None  # entry 0 transparent
    _, _, data = images.decode(png(packed, w, h, depth, 3, palette=palette, trns=trns))
    r, g, b = _unpack(data.reshape(h, w))
    expect = palette[idx].astype(np.int64)
    if trns:
        expect[idx == 0] = 0
    assert np.array_equal(np.stack([r, g, b], -1), expect)
    _, _, grey = images.decode(png(packed, w, h, depth, 0))
    level = idx * (255 // (n - 1))
    assert np.array_equal(grey.reshape(h, w) & 255, level)


@pytest.mark.parametrize("sub,restart,bound", [(1, 0, 4), (1, 5, 4), (2, 3, 12)])
def test_baseline_jpeg_round_trip(sub, restart, bound):
    h, w = 45, 70  # partial MCUs on both edges
    rgb = smooth_image(h, w, 3 + sub)
    data = encode_jpeg(rgb, sub=sub, restart=restart)
    ww, hh, px = images.decode(data)
    assert (ww, hh) == (w, h)
    r, g, b = _unpack(px.reshape(h, w).astype(np.int64))
    got = np.stack([r, g, b], -1)
    err = np.abs(got - rgb.astype(np.int64))
    assert err.max() <= bound, err.max()
    assert err.mean() <= 1.5, err.mean()


def test_zigzag_order_is_the_standard_one():
    """T.81 figure A.6: coded position k -> row-major index in the block."""
    assert images.ZIGZAG[:16].tolist() == [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5]
    assert images.ZIGZAG[-6:].tolist() == [61, 54, 47, 55, 62, 63]
    assert sorted(images.ZIGZAG.tolist()) == list(range(64))


def _block_edge_ratio(px, w, h):
    """Mean horizontal gradient across 8-pixel block edges over the mean inside blocks: about 1 for
    a correctly decoded natural image; a transposed zig-zag or inverse DCT gives 1.5 and more."""
    g = ((px >> 8) & 255).reshape(h, w).astype(np.float64)
    d = np.abs(np.diff(g, axis=1))
    cols = np.arange(w - 1)
    return d[:, cols % 8 == 7].mean() / d[:, cols % 8 != 7].mean()


def test_progressive_jpeg_is_refused():
    with pytest.raises(ValueError):
        images.decode(b"\xff\xd8\xff\xc2\x00\x0b\x08\x00\x08\x00\x08\x01\x01\x11\x00\xff\xd9")


@pytest.mark.skipif(not TEX.exists(), reason="reference textures not available")
def test_reference_textures_decode():
    w, h, d = images.load(TEX / "Texture_2.png")
    assert (w, h, d.size) == (512, 512, 512 * 512)
    w, h, d = images.load(TEX / "bricks2_normal.jpg")
    assert (w, h) == (512, 512)
    b = d & 255
    assert b.mean() > 200  # a tangent-space normal map points mostly along +z
    # Its texels encode unit vectors (2 c / 255 - 1): 0.007 mean deviation from length 1 when
    # decoded correctly, 0.024 with a transposed zig-zag, 0.3 with a transposed inverse DCT.
    n = np.stack([((d >> s) & 255) / 255.0 * 2.0 - 1.0 for s in (16, 8, 0)], -1)
    assert np.abs(np.linalg.norm(n, axis=-1) - 1.0).mean() < 0.012
    w, h, d = images.load(TEX / "bricks2.jpg")  # 2 x 2 chroma subsampling
    assert _block_edge_ratio(d, w, h) < 1.2
