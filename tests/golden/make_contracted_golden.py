"""Generate tests/golden/contracted_golden.npz from the reference's own GPU
build with nvcc's default contraction (oracle/_ref/ref_mandelbrot.cubin,
built by oracle/build_ref.sh), so that the CPU suite can check the oracle's
contracted restatement (ARITH_CONTRACTED) against the reference itself.

Needs a GB300 and the reference cubins.  Renders, with the Java host's launch
shape, seeded fractalRenderMain views (binary32 and binary64, several maxSS,
adaptive sampling on and off) and fractalRenderAdvanced zoom steps (sample
reuse, zooming in and out, the blend near the zoom centre) whose previous
frame is the same build's main frame; saves every pixel record.

    python tests/golden/make_contracted_golden.py [output.npz]
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "chaos-ultra_gb300"))

OUT = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "contracted_golden.npz")
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_mandelbrot.cubin")

# (name, centre, zoom (plane height), w, h, maxIter, maxSS, flags, binary64)
MAIN = [
    ("m_f32_ss1", (-0.748, 0.1), 0.0014, 64, 48, 600, 1.0, 0, False),
    ("m_f32_ss5", (-0.235125, 0.827215), 4.0e-5, 56, 40, 900, 5.0, 1, False),
    ("m_f64_ss1", (-0.74364388703715, 0.13182590420531), 2e-10, 64, 48, 3000, 1.0, 0, True),
    ("m_f64_ss7", (-0.925, 0.266), 0.032, 48, 40, 800, 7.0, 1, True),
    ("m_f64_ss17", (0.3004395381261789, -0.5705143370804123), 1e-9, 40, 32, 2000, 17.0, 1, True),
]
# (name, centre, zoom, w, h, maxIter, maxSS, focus, zoom in, flags, binary64)
ADVANCED = [
    ("a_f32_in", (-0.748, 0.1), 0.0014, 64, 40, 600, 3.0, (20, 25), True, 8 | 16 | 32 | 1, False),
    ("a_f32_out", (0.285, 0.01), 0.07, 64, 40, 900, 3.9, (50, 9), False, 8 | 16, False),
    ("a_f64_in", (-0.74364388703715, 0.13182590420531), 1e-7, 64, 40, 1500, 4.0, (30, 10), True, 8 | 16 | 32 | 1,
     True),
    ("a_f64_out", (-0.925, 0.266), 0.032, 48, 40, 800, 3.0, (5, 30), False, 8 | 16 | 1, True),
]


def main():
    import torch

    from tests.gpu_util import Driver, advanced_params, java_grid, main_params, pitched, read_pixels, upload_pixels
    from tests.test_gpu_reference_mode import rect_for, zoom_at

    torch.cuda.set_device(0)
    torch.zeros(1, device="cuda:0")
    drv = Driver()
    mod = drv.load(CUBIN)
    out, meta = {}, {"main": [], "advanced": []}
    try:
        drv.write_constant(mod, "VISUALIZE_SAMPLE_COUNT", b"\0")

        def main_frame(dbl, w, h, rect, mi, mss, flags):
            fn = drv.function(mod, "fractalRenderMainDouble" if dbl else "fractalRenderMainFloat")
            buf, pitch = pitched(torch, w, h)
            drv.launch(fn, java_grid(w, h)[0], (32, 32), main_params(buf.data_ptr(), pitch, w, h, rect, mi, mss, flags,
                                                                     dbl))
            return read_pixels(buf, w)

        for name, c, zoom, w, h, mi, mss, flags, dbl in MAIN:
            rect = rect_for(c, zoom, w, h)
            if not dbl:
                rect = tuple(float(v) for v in np.float32(rect))
            out[name] = main_frame(dbl, w, h, rect, mi, mss, flags).view(np.uint8).reshape(h, w, 16)
            meta["main"].append({"name": name, "rect": list(rect), "w": w, "h": h, "max_iter": mi, "max_ss": mss,
                                 "flags": flags, "dbl": dbl})
        for name, c, zoom, w, h, mi, mss, focus, into, flags, dbl in ADVANCED:
            old = rect_for(c, zoom, w, h)
            new = zoom_at(old, focus, w, h, into=into)
            if not dbl:
                old = tuple(float(v) for v in np.float32(old))
                new = tuple(float(v) for v in np.float32(new))
            prev = main_frame(dbl, w, h, old, mi, mss, 1)
            inbuf, in_pitch = upload_pixels(torch, prev)
            fn = drv.function(mod, "fractalRenderAdvancedDouble" if dbl else "fractalRenderAdvancedFloat")
            buf, pitch = pitched(torch, w, h)
            drv.launch(fn, java_grid(w, h)[0], (32, 32),
                       advanced_params(buf.data_ptr(), pitch, w, h, new, mi, mss, flags, old, inbuf.data_ptr(),
                                       in_pitch, focus, dbl))
            out[name + "_prev"] = prev.view(np.uint8).reshape(h, w, 16)
            out[name] = read_pixels(buf, w).view(np.uint8).reshape(h, w, 16)
            meta["advanced"].append({"name": name, "old": list(old), "new": list(new), "w": w, "h": h, "max_iter": mi,
                                     "max_ss": mss, "focus": list(focus), "flags": flags, "dbl": dbl})
    finally:
        drv.unload(mod)
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **out)
    print(OUT, sum(v.nbytes for v in out.values()))


if __name__ == "__main__":
    main()
