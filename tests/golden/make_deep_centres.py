"""Write chaos-ultra_gb300/chaos_gb300/data/deep_centres.json: the centre of the perturbation deep-zoom
workload (1920x1080, spans 1e-60 and 1e-200, maxIter 100000), a seeded point
on the Mandelbrot set boundary as a 1024-bit fixed-point value.

The centre is a Misiurewicz point: c whose critical orbit is strictly
preperiodic, z_{k+q}(c) = z_k(c) with preperiod exactly k and period exactly
q.  Such points lie on the boundary and the set is asymptotically self-similar
around them, so a view shows structure at every depth.  (Bisection along a ray
from the main cardioid, the centre of the binary64 workloads, ends next to the
cardioid where the escape count is flat below about 1e-120: a 1e-200 window
there is uniformly maxIter.)

Seeded search: for attempt = 0, 1, ... draw k in [8, 16], q in [1, 3] and a
start point uniform in [-2, 0.5] x [-1.2, 1.2]; run Newton's method on
g(c) = z_{k+q}(c) - z_k(c) at 1150 bits; accept the first root where Newton
converged below 2^-1080, the preperiod is exactly k (z_{k-1+q} != z_{k-1}) and
the period exactly q (z_{k+d} != z_k for proper divisors d of q).  Needs
mpmath; the result is committed so renders do not need it.

    python tests/golden/make_deep_centres.py
"""
import json
import os
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(os.path.dirname(HERE)), "chaos-ultra_gb300")
sys.path.insert(0, PKG)
DATA = os.path.join(PKG, "chaos_gb300", "data")

SEED, BITS, PREC = 3, 1024, 1150


def g(mp, c, k, q):
    """z_{k+q}(c) - z_k(c) and its derivative in c."""
    z = dz = mp.mpc(0)
    zk = dzk = None
    for n in range(1, k + q + 1):
        dz = 2 * z * dz + 1
        z = z * z + c
        if n == k:
            zk, dzk = z, dz
    return z - zk, dz - dzk


def search(seed=SEED, attempts=64):
    import mpmath as mp
    import numpy as np
    mp.mp.prec = PREC
    rng = np.random.default_rng(seed)
    tiny, small = mp.mpf(2) ** -1080, mp.mpf(2) ** -900
    for attempt in range(attempts):
        k, q = int(rng.integers(8, 17)), int(rng.integers(1, 4))
        sx, sy = float(rng.uniform(-2.0, 0.5)), float(rng.uniform(-1.2, 1.2))
        c = mp.mpc(sx, sy)
        converged = False
        for _ in range(400):
            f, df = g(mp, c, k, q)
            st = f / df
            c -= st
            if abs(c) > 4:
                break
            if abs(st) < tiny:
                converged = True
                break
        if not converged:
            continue
        if abs(g(mp, c, k - 1, q)[0]) < small:
            continue  # smaller preperiod
        if any(abs(g(mp, c, k, d)[0]) < small for d in range(1, q) if q % d == 0):
            continue  # smaller period
        return {"seed": seed, "attempt": attempt, "preperiod": k, "period": q, "start": [sx, sy], "c": c}
    raise RuntimeError("no Misiurewicz point found")


def to_hex(mp, v, bits=BITS):
    """mpmath real -> "[-]I.hex" with `bits` fraction bits, truncated."""
    from chaos_gb300.api import to_hex_fixed
    sign, man, exp, _ = mp.mpf(v)._mpf_
    return to_hex_fixed((-1) ** sign * Fraction(int(man)) * Fraction(2) ** exp, bits)


def main():
    import mpmath as mp
    r = search()
    c = r.pop("c")
    r.update({"bits": BITS, "center_x": to_hex(mp, c.real), "center_y": to_hex(mp, c.imag),
              "approx": [float(c.real), float(c.imag)]})
    os.makedirs(DATA, exist_ok=True)
    with open(os.path.join(DATA, "deep_centres.json"), "w") as f:
        json.dump(r, f, indent=1)
        f.write("\n")
    print(r["attempt"], r["preperiod"], r["period"], r["approx"])


if __name__ == "__main__":
    main()
