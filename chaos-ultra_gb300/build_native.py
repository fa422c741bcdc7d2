"""Build the native parts of chaos_gb300 for sm_103a, in-tree.

Outputs (git-ignored):
  lib/libchaos_gb300.so                 the C-ABI library (include/chaos_gb300.h)
  cudaKernels/<fractal>.ptx             drop-in modules with the arithmetic of the
                                        reference's default build (contraction on)
  cudaKernels_parity/<fractal>.ptx      drop-in modules, every product/sum rounded
The drop-in files are cubin images; cuModuleLoad (which the Java host calls
with <cudaKernelsDir>/<fractal>.ptx) accepts cubin as well as PTX.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
FRACTALS = {"mandelbrot": 0, "julia": 1, "newton_wired": 2, "newton_generic": 3, "newton_iterations": 4}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(verbose=False, ptxas_info=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.join(HERE, "lib"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "cudaKernels"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "cudaKernels_parity"), exist_ok=True)
    exe = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "chaos_gb300.h"))
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    jobs = []
    objs = []
    for name in ("chaos_kernels", "chaos_api", "chaos_perturb", "chaos_noalloc", "chaos_batch", "chaos_serve",
                 "chaos_newton"):
        src = os.path.join(CSRC, name + ".cu")
        obj = os.path.join(BUILD, name + ".o")
        objs.append(obj)
        # the Newton modules' thrust::complex code is rounded operation by operation
        fmad = ["--fmad=false"] if name == "chaos_newton" else []
        if force or not _newer(obj, [src] + headers):
            jobs.append([exe, *ARCH, *COMMON, *extra, *fmad, "-Xcompiler", "-fPIC", "-c", src, "-o", obj])
    dropin = os.path.join(CSRC, "dropin_module.cu")
    for fractal, fid in FRACTALS.items():
        # cudaKernels: the arithmetic of the reference as nvcc builds it by
        # default; cudaKernels_parity: every product and sum rounded
        for sub, arith in (("cudaKernels", "chaos::ARITH_CONTRACTED"), ("cudaKernels_parity", "chaos::ARITH_PARITY")):
            out = os.path.join(HERE, sub, fractal + ".ptx")
            if force or not _newer(out, [dropin] + headers):
                # every contraction of the shared sampling / reuse / compose code is
                # spelled out in the source (intrinsics, which nvcc never fuses).
                # The Newton steps are thrust::complex expressions as in the
                # reference: in the default-build modules nvcc contracts them as it
                # contracts the reference's own (same compiler, same expressions)
                newton_default = fid >= 2 and sub == "cudaKernels"
                fmad = [] if newton_default else ["--fmad=false"]
                jobs.append([exe, *ARCH, *COMMON, *extra, *fmad, "-cubin", f"-DCHAOS_DROPIN_FRACTAL={fid}",
                             f"-DCHAOS_DROPIN_ARITH={arith}", dropin, "-o", out])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    lib = os.path.join(HERE, "lib", "libchaos_gb300.so")
    if force or not _newer(lib, objs):
        _run([exe, *ARCH, "-shared", *objs, "-o", lib, "-lcudart"])
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv, force="-f" in sys.argv))
