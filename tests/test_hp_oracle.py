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
