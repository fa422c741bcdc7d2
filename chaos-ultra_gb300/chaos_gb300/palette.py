"""Palettes (RGBA8 words, R in the low byte)."""
import numpy as np


def _rgba(r, g, b):
    # ImageHelpers.fromRGBtoRGBA: each channel shifted into place and masked to 8 bits
    return ((r << 0) & 0xFF) | ((g << 8) & 0xFF00) | ((b << 16) & 0xFF0000) | 0xFF000000


def default_palette():
    """The 1536-entry palette the reference builds when no palette file is given
    (ImageHelpers.createDefaultColorPalette, J/util/ImageHelpers.java:77-111)."""
    m, full = 256, 255
    p = []
    for i in range(0, m):
        p.append(_rgba(i, 0, min(full, full // 2 + i)))
    for i in range(m, 2 * m):
        p.append(_rgba(full, 0, full - i))
    for i in range(2 * m, 3 * m):
        p.append(_rgba(full, i, 0))
    for i in range(3 * m, 4 * m):
        p.append(_rgba(full - i, full, 0))
    for i in range(4 * m, 5 * m):
        p.append(_rgba(0, full, i))
    for i in range(5 * m, 6 * m):
        p.append(_rgba(0, full - i, full))
    return np.array(p, dtype=np.uint32)


def seeded_palette(n=256, seed=0):
    """n RGBA8 entries with uniform random R, G, B bytes and alpha 255."""
    rng = np.random.default_rng(seed)
    rgb = rng.integers(0, 256, size=(n, 3), dtype=np.uint32)
    return (rgb[:, 0] | (rgb[:, 1] << 8) | (rgb[:, 2] << 16) | np.uint32(0xFF000000)).astype(np.uint32)
