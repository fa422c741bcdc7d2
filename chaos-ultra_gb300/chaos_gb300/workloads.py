"""Seeded synthetic workloads of the benchmark configurations.

All inputs are generated from seeds (no datasets exist for this path):
boundary centres by bisection between a point inside the main cardioid and a
point on |c| = 2.5, palettes from uniform random bytes, jitter offsets from the
library's counter-based hash.
"""
import math
from fractions import Fraction

import numpy as np

from .api import to_hex_fixed
from .palette import seeded_palette


def _escapes(cx, cy, max_iter):
    x = y = 0.0
    for _ in range(max_iter):
        xx, yy = x * x, y * y
        if xx + yy >= 4.0:
            return True
        y = 2.0 * x * y + cy
        x = xx - yy + cx
    return False


def ray_endpoints(seed):
    """Seeded interior point of the main cardioid (c = mu/2 - mu^2/4, |mu| < 1)
    and a seeded point on |c| = 2.5."""
    rng = np.random.default_rng(seed)
    r, t, s = rng.uniform(0.3, 0.95), rng.uniform(0, 2 * math.pi), rng.uniform(0, 2 * math.pi)
    mu = complex(r * math.cos(t), r * math.sin(t))
    return mu / 2 - mu * mu / 4, complex(2.5 * math.cos(s), 2.5 * math.sin(s))


def boundary_point(seed, max_iter=20000, steps=200):
    """Bisection along the seeded ray until the binary64 interval collapses."""
    c_in, c_out = ray_endpoints(seed)
    for _ in range(steps):
        mid = (c_in + c_out) / 2
        if mid == c_in or mid == c_out:
            break
        if _escapes(mid.real, mid.imag, max_iter):
            c_out = mid
        else:
            c_in = mid
    return c_in.real, c_in.imag


def boundary_points(seeds, max_iter=4000, steps=64):
    """boundary_point for many seeds at once (numpy, vectorised over seeds)."""
    ends = [ray_endpoints(s) for s in seeds]
    cin = np.array([e[0] for e in ends], dtype=np.complex128)
    cout = np.array([e[1] for e in ends], dtype=np.complex128)
    for _ in range(steps):
        mid = (cin + cout) / 2
        x = np.zeros(len(mid))
        y = np.zeros(len(mid))
        alive = np.ones(len(mid), dtype=bool)
        for _ in range(max_iter):
            xx, yy = x * x, y * y
            alive &= (xx + yy) < 4.0
            if not alive.any():
                break
            y = np.where(alive, 2.0 * x * y + mid.imag, y)
            x = np.where(alive, xx - yy + mid.real, x)
        esc = ~alive
        cout = np.where(esc, mid, cout)
        cin = np.where(esc, cin, mid)
    return [(c.real, c.imag) for c in cin]


def deep_center(seed, bits=1024, max_iter=20000):
    """A deep-zoom centre as "[-]I.hex" strings with `bits` fraction bits: the
    boundary point of `seed` extended below its binary64 precision with seeded
    random bits."""
    cx, cy = boundary_point(seed, max_iter)
    rng = np.random.default_rng(seed + 12345)
    out = []
    for v in (cx, cy):
        low = Fraction(int.from_bytes(rng.bytes(bits // 8), "little"), 1 << bits) * Fraction(2) ** -60
        f = Fraction(v) + (low if v >= 0 else -low)
        out.append(to_hex_fixed(f, bits))
    return out[0], out[1]


def c4_viewports(seed=4, n=64):
    """Batched uneven launch: n Mandelbrot viewports, side log-uniform in
    [256, 2048] (multiple of 8), span log-uniform in [1e-12, 1e-3], maxIter
    log-uniform in [500, 50000], seeded boundary centres.  Returns dicts with
    width, height, span, max_iter, center, seed."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        side = int(round(math.exp(rng.uniform(math.log(256), math.log(2048))) / 8.0)) * 8
        span = 10.0 ** rng.uniform(-12, -3)
        mi = int(round(math.exp(rng.uniform(math.log(500), math.log(50000)))))
        specs.append({"width": side, "height": side, "span": span, "max_iter": mi, "seed": 100 * seed + k})
    centres = boundary_points([s["seed"] for s in specs])
    for s, c in zip(specs, centres):
        s["center"] = c
    return specs


def c4_palette(seed=4):
    return seeded_palette(256, seed=seed)


def deep_zoom_centre():
    """The perturbation deep-zoom centre (1920x1080, spans 1e-60 and 1e-200,
    maxIter 100000): a seeded Misiurewicz point as 1024-bit "[-]I.hex" strings,
    with its preperiod and period (data/deep_centres.json, written by
    tests/golden/make_deep_centres.py)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "deep_centres.json")) as f:
        return json.load(f)
