"""Build the oracle (test infrastructure only).

  oracle/_build/libchaos_oracle.so   the CPU restatement, oracle/chaos_oracle.c
  oracle/_ref/...                    the reference's own code (oracle/build_ref.sh),
                                     built when the reference checkout (or an
                                     earlier build-directory copy) is present
"""
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")


def _run(cmd, env=None):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _elf_machine(path):
    """e_machine of an ELF file, or None."""
    try:
        with open(path, "rb") as f:
            h = f.read(20)
        if h[:4] != b"\x7fELF":
            return None
        return int.from_bytes(h[18:20], "little")
    except OSError:
        return None


def _host_machine():
    return {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.isdir(os.path.join(d, "include")):
            return os.path.join(d, "include")
    return "/usr/local/cuda/include"


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "chaos_oracle.c")
    src_cpp = os.path.join(HERE, "newton_oracle.cpp")
    out = os.path.join(BUILD, "libchaos_oracle.so")
    newest = max(os.path.getmtime(src), os.path.getmtime(src_cpp))
    if not (os.path.exists(out) and os.path.getmtime(out) >= newest and _elf_machine(out) == _host_machine()):
        # fma()/fmaf() are exact on either CPU; -mfma only makes them one
        # instruction on x86-64 (-ffp-contract=off still forbids contraction).
        isa = ["-mfma"] if platform.machine() == "x86_64" else []
        inc = _cuda_include()
        obj_c = os.path.join(BUILD, "chaos_oracle.o")
        obj_cpp = os.path.join(BUILD, "newton_oracle.o")
        _run([os.environ.get("CC", "gcc"), "-O2", "-ffp-contract=off", "-fno-fast-math", *isa, "-fopenmp", "-fPIC",
              "-std=c11", "-c", src, "-o", obj_c])
        # thrust::complex on the host, from the CUDA toolkit's headers
        _run([os.environ.get("CXX", "g++"), "-O2", "-ffp-contract=off", "-fno-fast-math", *isa, "-fPIC",
              "-std=c++17", "-I", inc, "-I", os.path.join(inc, "cccl"), "-c", src_cpp, "-o", obj_cpp])
        _run([os.environ.get("CXX", "g++"), "-shared", "-fopenmp", obj_c, obj_cpp, "-o", out, "-lm"])
    return out


def reference_root():
    """Where the reference checkout is read from: $REFERENCE_ROOT, else a
    chaos-ultra checkout named `reference` beside this repository."""
    return os.environ.get("REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT_DIR), "reference")


def build_reference():
    """Run oracle/build_ref.sh when the reference sources are reachable.

    Returns the path of oracle/_ref/libchaos_ref.so, or None.  The cubins are
    only rebuilt where nvcc exists; the host library is rebuilt when it is
    missing or built for another CPU architecture."""
    ref_root = reference_root()
    have_src = os.path.isdir(os.path.join(ref_root, "src", "main", "cuda")) or os.path.exists(
        os.path.join(REF_OUT, "src", "fractalRendererGeneric.cu"))
    if not have_src:
        return None
    lib = os.path.join(REF_OUT, "libchaos_ref.so")
    cubins = [os.path.join(REF_OUT, f"ref_{f}{s}.cubin")
              for f in ("mandelbrot", "julia", "newton_wired", "newton_generic", "newton_iterations")
              for s in ("", "_nofma")]
    need_host = _elf_machine(lib) != _host_machine()
    need_cubin = not all(os.path.exists(c) for c in cubins)
    if need_host or need_cubin or os.path.isdir(os.path.join(ref_root, "src")):
        env = dict(os.environ)
        if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
            env["SKIP_CUBIN"] = "1"
        elif not shutil.which("nvcc"):
            env["NVCC"] = "/usr/local/cuda/bin/nvcc"
        if not need_cubin and not os.path.isdir(os.path.join(ref_root, "src")):
            env["SKIP_CUBIN"] = "1"
        env["REFERENCE_ROOT"] = ref_root
        _run(["sh", os.path.join(HERE, "build_ref.sh")], env=env)
    return lib if os.path.exists(lib) else None


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference())
