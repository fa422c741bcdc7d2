"""The oracle's multi-word direct iteration against mpmath (committed golden
vectors, tests/golden/make_hp_golden.py)."""
import json
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "hp_golden.json")


def test_hp_oracle_matches_mpmath(oracle):
    cases = json.load(open(GOLDEN))["cases"]
    assert len(cases) >= 40
    bad = []
    for c in cases:
        n, _ = oracle.hp_escape(c["cx"], c["cy"], c["dcx"], c["dcy"], c["bits"], c["max_iter"])
        if n != c["count"]:
            bad.append((c, n))
    assert not bad, bad[:3]


def test_hex_fixed_roundtrip(native):
    from fractions import Fraction

    import chaos_gb300 as cg
    assert cg.to_hex_fixed(Fraction(-3, 4), 8) == "-0.c0"
    assert cg.to_hex_fixed(1.5, 4) == "1.8"
    assert cg.to_hex_fixed(Fraction(1, 3), 16) == "0.5555"


def test_orbit_argument_checks(native):
    import chaos_gb300 as cg
    for args in (("0.8", "0.zz", 128, 100), ("0.8", "0.0", 32, 100), ("0.8", "0.0", 128, 0), ("9.0", "0.0", 128, 10)):
        with pytest.raises(cg.ChaosError) as e:
            cg.Orbit(*args)
        assert e.value.code == 1


def test_deep_centre_is_a_misiurewicz_point(oracle):
    """The committed deep-zoom centre: z_{k+q} = z_k at 1100 bits with preperiod
    exactly k (mpmath), and the oracle sees structure in a 1e-200 window."""
    mp = pytest.importorskip("mpmath")
    import numpy as np

    from chaos_gb300.workloads import deep_zoom_centre
    d = deep_zoom_centre()
    assert d["bits"] == 1024 and len(d["center_x"].split(".")[1]) == 256
    mp.mp.prec = 1100

    def hexval(h):
        neg = h.startswith("-")
        ip, fp = h.lstrip("-").split(".")
        v = mp.mpf(int(ip)) + mp.mpf(int(fp, 16)) / mp.mpf(16) ** len(fp)
        return -v if neg else v

    c = mp.mpc(hexval(d["center_x"]), hexval(d["center_y"]))
    k, q = d["preperiod"], d["period"]
    zs = [mp.mpc(0)]
    for _ in range(k + q):
        zs.append(zs[-1] ** 2 + c)
    assert abs(zs[k + q] - zs[k]) < mp.mpf(2) ** -1000
    assert abs(zs[k - 1 + q] - zs[k - 1]) > mp.mpf(2) ** -20
    ps = 1e-200 / 1920
    xs, ys = np.meshgrid((np.arange(16) + 0.5 - 8) * 120 * ps, -(np.arange(9) + 0.5 - 4.5) * 120 * ps)
    counts, _ = oracle.hp_escape_batch(d["center_x"], d["center_y"], xs.ravel(), ys.ravel(), 768, 100000)
    assert len(np.unique(counts)) >= 8 and counts.max() < 100000
