"""Generate tests/golden/reference_golden.json from the reference's own code.

Runs the reference's src/main/cuda/fractals/{mandelbrot,julia}.cu, host-built
by oracle/build_ref.sh (oracle/_ref/libchaos_ref.so), on seeded inputs and
records its outputs.  The JSON is committed; the tests check the oracle
(oracle/chaos_oracle.c) against it on any machine, with or without the
reference checkout.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "chaos-ultra_gb300"))

from oracle import build_oracle  # noqa: E402
from oracle.oracle import Reference, c1_grid  # noqa: E402
from chaos_gb300.palette import default_palette  # noqa: E402

# Julia constants from the reference's presets (ModuleJulia.java:47-53, PresenterFX.java:294-334)
JULIA_C = [(-0.4, 0.6), (-0.8, 0.156), (0.285, 0.01), (-1.77578, 0.0), (-1.77578, 0.0035)]
# Premade Mandelbrot views M1-M5 (PresenterFX.java:244-292): centre, zoom (plane height), maxIterations
VIEWS = [(-0.748, 0.1, 0.0014, 1600), (-0.235125, 0.827215, 4.0e-5, 1600), (-0.925, 0.266, 0.032, 1600),
         (-0.57675236, 0.4625193, 0.029995363, 1600), (-0.551042868375875, 0.62714332109057, 8.00592947491907e-09,
                                                        3000)]


def main():
    if build_oracle.build_reference() is None:
        raise SystemExit("reference sources not available")
    ref = Reference()
    rng = np.random.default_rng(20261203)
    out = {"generator": "tests/golden/make_golden.py", "source": "reference computeFractal/colorize, host build"}

    # C1: 1024^2 pixel centres of [-2,1]x[-1.5,1.5], maxIter 1000
    w, h, x0, y0, dx, dy, mi = c1_grid()
    c1 = {"w": w, "h": h, "x0": x0, "y0": y0, "dx": dx, "dy": dy, "max_iter": mi}
    for dbl, tag in ((0, "f32"), (1, "f64")):
        total, counts = ref.grid(dbl, w, h, x0, y0, dx, dy, mi)
        c1[f"total_{tag}"] = int(total)
        c1[f"interior_{tag}"] = int((counts == mi).sum())
        c1[f"sha256_{tag}"] = hashlib.sha256(counts.astype("<u4").tobytes()).hexdigest()
        c1[f"crop_{tag}"] = counts[300:332, 600:632].tolist()
    out["c1"] = c1

    # Mandelbrot points: uniform over the set's neighbourhood and around the premade views
    pts = []
    for _ in range(256):
        pts.append((float(rng.uniform(-2.1, 0.7)), float(rng.uniform(-1.3, 1.3)), 1000))
    for cx, cy, zoom, mi in VIEWS:
        for _ in range(64):
            pts.append((cx + zoom * float(rng.uniform(-0.8, 0.8)), cy + zoom * float(rng.uniform(-0.5, 0.5)), mi))
    mand = []
    for x, y, mi in pts:
        mand.append({"x": x, "y": y, "max_iter": mi, "f32": ref.mandelbrot(0, mi, np.float32(x), np.float32(y)),
                     "f64": ref.mandelbrot(1, mi, x, y)})
    out["mandelbrot_points"] = mand

    jul = []
    for c in JULIA_C:
        for _ in range(64):
            x, y = float(rng.uniform(-1.6, 1.6)), float(rng.uniform(-1.0, 1.0))
            jul.append({"c": list(c), "x": x, "y": y, "max_iter": 900,
                        "f32": ref.julia(0, 900, np.float32(x), np.float32(y), c),
                        "f64": ref.julia(1, 900, x, y, c)})
    out["julia_points"] = jul

    pal = default_palette()
    vals = [float(v) for v in np.concatenate([np.arange(0, 40, 0.25), rng.uniform(0, 5000, 64)])]
    out["default_palette_sha256"] = hashlib.sha256(pal.astype("<u4").tobytes()).hexdigest()
    out["colorize_default_palette"] = [{"value": v, "rgba": int(ref.colorize(pal, v))} for v in vals]

    # Newton modules: default parameters and the other set the reference suggests
    # (ModuleNewtonGeneric.java:67-74), coefficients stored c0..c3
    newton_params = [
        {"roots": [1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378], "coefficients": [-1, 0, 0, 1], "magnifier": 11},
        {"roots": [-1.7692923542386314, 0, 0.884646177119315707620204, 0.589742805022205501647280,
                   0.884646177119315707, -0.589742805022205501], "coefficients": [2, -2, 0, 1], "magnifier": 7},
    ]
    newton = []
    for pi, prm in enumerate(newton_params):
        ref.newton_set(prm["roots"], prm["coefficients"], prm["magnifier"])
        for kind in (2, 3, 4):
            for _ in range(48):
                x, y = float(rng.uniform(-2, 2)), float(rng.uniform(-1.5, 1.5))
                newton.append({"params": pi, "kind": kind, "x": x, "y": y, "max_iter": 200,
                               "f32": ref.newton(kind, 0, 200, np.float32(x), np.float32(y)),
                               "f64": ref.newton(kind, 1, 200, x, y)})
    out["newton_params"] = newton_params
    out["newton_points"] = newton
    ref.newton_set(newton_params[0]["roots"], newton_params[0]["coefficients"], 11)
    out["newton_colorize"] = [{"kind": k, "value": float(v), "rgba": int(ref.newton_colorize(k, pal, float(v)))}
                              for k in (2, 3, 4) for v in list(range(0, 6)) + [17.0, 99.0, 1234.0]]

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
