"""Generate tests/golden/hp_golden.json: high-precision escape counts from mpmath.

Pins the oracle's multi-word direct iteration (oracle/chaos_oracle.c,
orc_hp_escape), the reference the deep-zoom tiers are judged against.  Points:
offsets from three centres -- the plain-workload boundary centre at span 1e-10
and a 1024-bit extension of it at spans 1e-60 and 1e-200 (seeded low bits).

    python tests/golden/make_hp_golden.py
"""
import json
import os
import sys
from fractions import Fraction

import mpmath
import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "chaos-ultra_gb300"))

import bench  # noqa: E402
from chaos_gb300 import to_hex_fixed  # noqa: E402


def hp_count(cx, cy, max_iter):
    zx = zy = mpmath.mpf(0)
    for i in range(max_iter):
        xx, yy = zx * zx, zy * zy
        if xx + yy >= 4:
            return i
        zy = 2 * zx * zy + cy
        zx = xx - yy + cx
    return max_iter


def main():
    rng = np.random.default_rng(99)
    cx0, cy0 = bench.boundary_point(bench.WORKLOAD_SEED)
    cases = []
    ext = bench.deep_center(bench.WORKLOAD_SEED, 1024)
    plan = [("boundary", 1e-10, 256, 20000, 12), ("boundary-1024", 1e-60, 384, 4000, 6),
            ("boundary-1024", 1e-200, 832, 3000, 4),
            # c = i: a Misiurewicz point (preperiodic, on the boundary) whose
            # neighbourhood keeps structure at every depth
            ("misiurewicz-i", 1e-60, 384, 3000, 12), ("misiurewicz-i", 1e-200, 832, 3000, 12)]
    for centre, span, bits, max_iter, n in plan:
        if centre == "boundary":
            hx, hy = to_hex_fixed(Fraction(cx0), bits), to_hex_fixed(Fraction(cy0), bits)
        elif centre == "misiurewicz-i":
            hx, hy = "0.0", "1.0"
        else:
            hx, hy = ext
        mpmath.mp.prec = bits + 64
        def parse(h):
            neg = h.startswith("-")
            ip, fr = h.lstrip("-").split(".")
            v = mpmath.mpf(int(ip)) + mpmath.mpf(int(fr, 16)) / mpmath.mpf(2) ** (4 * len(fr))
            return -v if neg else v
        cxm, cym = parse(hx), parse(hy)
        ps = span / 1920
        for _ in range(n):
            dx = float(rng.uniform(-960, 960) * ps)
            dy = float(rng.uniform(-540, 540) * ps)
            cnt = hp_count(cxm + mpmath.mpf(dx), cym + mpmath.mpf(dy), max_iter)
            cases.append({"centre": centre, "cx": hx, "cy": hy, "dcx": dx, "dcy": dy, "bits": bits,
                          "max_iter": max_iter, "span": span, "count": cnt})
            print(span, cnt, flush=True)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hp_golden.json")
    with open(path, "w") as f:
        json.dump({"generator": "tests/golden/make_hp_golden.py", "source": "mpmath 1.3 at bits+64 precision",
                   "cases": cases}, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
