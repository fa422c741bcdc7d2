"""The integer-unit binary64 subtraction used by the rounded binary64 escape
step (chaos-ultra_gb300/csrc/chaos_intarith.cuh), built for the host and
checked against the host's own subtraction on seeded operand classes
(tests/intarith_check.cpp): every result not handed back to the
floating-point unit must be bit-identical."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "chaos-ultra_gb300", "csrc")


def test_sub_nonneg_bits_matches_host_subtraction(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "intarith_check")
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-I", CSRC, "-o", exe,
                    os.path.join(ROOT, "tests", "intarith_check.cpp")], check=True)
    out = subprocess.run([exe, "6000000"], capture_output=True, text=True)
    n, flagged, wrong = (int(v) for v in out.stdout.split()[-3:])
    assert out.returncode == 0 and wrong == 0, out.stdout
    assert n == 6000000
    assert flagged < n // 10  # only subnormal, zero-pair and special classes go back


@pytest.mark.gpu
def test_sub_nonneg_bits_matches_device_subtraction(cuda, tmp_path):
    """The same routine built for sm_103a against the GPU's own __dsub_rn."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "intarith_gpu_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I", CSRC, "-o", exe,
                    os.path.join(ROOT, "tests", "intarith_gpu_check.cu")], check=True)
    out = subprocess.run([exe, str(1 << 26)], capture_output=True, text=True, timeout=120)
    n, flagged, wrong = (int(v) for v in out.stdout.split()[-3:])
    assert out.returncode == 0 and wrong == 0, out.stdout
    assert n == 1 << 26 and flagged < n // 10
