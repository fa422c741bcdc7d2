"""The composed-block bound of the perturbation kernels, restated on the CPU.

The perturbation kernels (csrc/chaos_perturb.cu) replace 16 or 64 steps
d <- (2 Z_j + d) d + dc by one composed linear map d <- P d + Q dc when the
exponent of max(|d|, |dc|) (componentwise) is at most a per-index bound the
host derives from |Z_j| and the block's partial products:

    bound_L(m) = floor(log2(rho) / 2 - slack),
    rho = min_{j = m..m+L} |Z_j|^2 / (2 (|P_(m->j)|^2 + |Q_(m->j)|^2)),

slack 25.5 for binary32 differences and 54.5 for binary64 ones, and no bound
where a test could fire inside the block (|Z_j|^2 >= 3.99 or < 2^-98).  The
premise is that under the bound the quadratic term of every step in the block
stays below the arithmetic's rounding: |d_j| <= 2^-p |Z_j| (p = 24, 53), so
|d_j^2| <= 2^-(p+1) |2 Z_j d_j|.  This test restates the bound for the
deep-zoom centre's orbit and checks the premise by iterating the full step
from offsets at the bound (the largest the kernels accept), in random
directions, at every index that has one."""
import math

import numpy as np
import pytest

MAX_STEPS = 1000  # the centre's 1088-bit orbit leaves |z| < 2 after ~930


def centre_orbit():
    mp = pytest.importorskip("mpmath")
    from chaos_gb300.workloads import deep_zoom_centre
    d = deep_zoom_centre()
    mp.mp.prec = 1100

    def parse(s):
        neg = s.startswith("-")
        ip, fp = s.lstrip("-").split(".")
        v = mp.mpf(int(ip, 16)) + mp.mpf(int(fp, 16)) / mp.mpf(16) ** len(fp)
        return -v if neg else v

    cx, cy = parse(d["center_x"]), parse(d["center_y"])
    zx = zy = mp.mpf(0)
    z = [(0.0, 0.0)]
    for _ in range(MAX_STEPS):
        zx, zy = zx * zx - zy * zy + cx, 2 * zx * zy + cy
        z.append((float(zx), float(zy)))
        if not (z[-1][0] ** 2 + z[-1][1] ** 2 < 4.0):
            break
    return np.array(z)


def bounds(z, slack, event):
    """(bound16, bound64) per index, None where no block may start: the
    restatement of the host's composition (compose_blocks)."""
    n = len(z)
    last = n - 1
    zz = z[:, 0] ** 2 + z[:, 1] ** 2
    ev = [event(j) for j in range(n)]
    out16, out64 = [None] * n, [None] * n

    def lim(rho):
        if not (rho > 0.0) or not math.isfinite(rho):
            return None
        v = math.floor(0.5 * math.log2(rho) - slack)
        return None if v < -127 else min(127, v)

    for m in range(0, n - 16):
        px, py, qx, qy = 1.0, 0.0, 0.0, 0.0
        ok16 = m + 16 < last and zz[m] > 0
        ok64 = m + 64 < last and zz[m] > 0
        rho = rho16 = math.inf
        for j in range(m, min(m + 65, n)):
            if j > m and ev[j]:
                if j <= m + 16:
                    ok16 = False
                ok64 = False
            if not ok64 and j > m + 16:
                break
            rho = min(rho, zz[j] / (2.0 * (px * px + py * py + qx * qx + qy * qy)))
            if j == m + 16:
                rho16 = rho
                if not ok64:
                    break
            if j == m + 64:
                ok64 = ok64 and 2.0 * (px * px + py * py + qx * qx + qy * qy) <= 2.0 ** 200
                break
            ax, ay = 2 * z[j, 0], 2 * z[j, 1]
            px, py = ax * px - ay * py, ax * py + ay * px
            qx, qy = ax * qx - ay * qy + 1.0, ax * qy + ay * qx
        out16[m] = lim(rho16) if ok16 else None
        out64[m] = lim(rho) if ok64 else None
    return out16, out64


def worst_ratio(z, m, length, e_max, rng, tries=4):
    """max over steps j of the block of |d_j| / |Z_j|, starting from offsets
    whose larger component has exponent e_max (the largest the bound admits)."""
    worst = 0.0
    for _ in range(tries):
        mag = 2.0 ** e_max * rng.uniform(1.0, 2.0, size=4) * rng.choice([-1.0, 1.0], size=4)
        mag[rng.integers(0, 4, size=2)] *= rng.uniform(0.0, 1.0, size=2)  # not all components at the top
        dx, dy, cx, cy = mag
        for j in range(m, m + length):
            r = math.hypot(dx, dy) / math.hypot(z[j, 0], z[j, 1])
            worst = max(worst, r)
            ax, ay = 2 * z[j, 0] + dx, 2 * z[j, 1] + dy
            dx, dy = ax * dx - ay * dy + cx, ax * dy + ay * dx + cy
    return worst


@pytest.mark.parametrize("p,slack", [(24, 25.5), (53, 54.5)])
def test_block_bound_keeps_the_quadratic_term_below_rounding(p, slack):
    z = centre_orbit()
    assert len(z) > 500
    if p == 24:
        z = z.astype(np.float32).astype(np.float64)  # the binary32 orbit those kernels read
    r2 = z[:, 0] ** 2 + z[:, 1] ** 2

    def event(j):
        return not (r2[j] < 3.99) or r2[j] < 2.0 ** -98

    b16, b64 = bounds(z, slack, event)
    valid16 = [m for m, b in enumerate(b16) if b is not None]
    valid64 = [m for m, b in enumerate(b64) if b is not None]
    # most indices of this orbit admit blocks, with bounds near 2^-p / |P|
    assert len(valid16) > 0.9 * (len(z) - 17) and len(valid64) > 0.8 * (len(z) - 65)
    assert all(b <= -(p + 1) for b in b16 if b is not None)  # never beyond 2^-p |Z_m|
    rng = np.random.default_rng(7)
    for length, bound, valid in ((16, b16, valid16), (64, b64, valid64)):
        for m in valid[:: max(1, len(valid) // 120)]:
            worst = worst_ratio(z, m, length + 1, bound[m], rng)
            assert worst <= 2.0 ** -p, (length, m, bound[m], math.log2(worst))


def test_no_block_spans_an_event():
    """Where a block would pass an index at which a test can fire (|Z_j|^2 at
    3.99 or more, below 2^-98) or reach the orbit's end, no bound is set."""
    z = centre_orbit().astype(np.float32).astype(np.float64)
    r2 = z[:, 0] ** 2 + z[:, 1] ** 2
    planted = 300  # plant an event in a copy of the orbit (the orbit itself has none there)
    zp = z.copy()
    zp[planted] = (1.999, 0.0)
    r2p = zp[:, 0] ** 2 + zp[:, 1] ** 2

    def event(j):
        return not (r2p[j] < 3.99) or r2p[j] < 2.0 ** -98

    b16, b64 = bounds(zp, 25.5, event)
    for m in range(planted - 16, planted):
        assert b16[m] is None, m
    for m in range(planted - 64, planted):
        assert b64[m] is None, m
    assert b16[planted] is not None or not (r2[planted + 1:planted + 17] < 3.99).all()
    n = len(zp)
    assert all(b is None for b in b16[n - 17:]) and all(b is None for b in b64[n - 65:])
