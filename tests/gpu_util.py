"""Helpers for the GPU tests: pitched device buffers (torch) and a ctypes
replay of the Java host's JCuda calls (cuModuleLoad, cuModuleGetFunction,
cuModuleGetGlobal + cudaMemcpy, cuLaunchKernel with a void** parameter array)."""
import ctypes as C

import numpy as np

from oracle.oracle import PIXEL_DTYPE

# The seven kernels FractalRenderingModule.initialize resolves
# (J/cudarenderer/FractalRenderingModule.java:91-97).
MODULE_KERNELS = ["fractalRenderMainFloat", "fractalRenderMainDouble", "fractalRenderAdvancedFloat",
                  "fractalRenderAdvancedDouble", "fractalRenderUnderSampled", "compose", "debug"]


def pitched(torch, w, h, pitch_align=512):
    """A pitched w x h buffer of 16-byte records, like cuMemAllocPitch(w*16, h, 16)."""
    pitch = ((16 * w + pitch_align - 1) // pitch_align) * pitch_align
    buf = torch.zeros((h, pitch), dtype=torch.uint8, device="cuda:0")
    return buf, pitch


def read_pixels(buf, w):
    """Device pitched buffer -> (h, w) numpy array of pixel records."""
    host = buf.cpu().numpy()
    return np.ascontiguousarray(host[:, : 16 * w]).view(PIXEL_DTYPE).reshape(host.shape[0], w)


def upload_pixels(torch, arr, pitch_align=512):
    h, w = arr.shape
    buf, pitch = pitched(torch, w, h, pitch_align)
    host = np.zeros((h, pitch), dtype=np.uint8)
    host[:, : 16 * w] = np.ascontiguousarray(arr).view(np.uint8).reshape(h, 16 * w)
    buf.copy_(torch.from_numpy(host))
    return buf, pitch


def same_pixels(a, b):
    """Field-wise equality of two pixel arrays (padding bytes ignored); returns mismatch mask."""
    m = np.zeros(a.shape, dtype=bool)
    for f in ("value", "weight", "is_reused", "weight_of_new_samples"):
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            m |= x.view(np.uint32) != y.view(np.uint32)
        else:
            m |= x != y
    return m


class Driver:
    """Minimal CUDA driver API through ctypes (the calls JCuda makes for the Java host)."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def load(self, path):
        mod = C.c_void_p()
        self._check(self.cu.cuModuleLoad(C.byref(mod), path.encode()), f"cuModuleLoad({path})")
        return mod

    def unload(self, mod):
        self._check(self.cu.cuModuleUnload(mod), "cuModuleUnload")

    def function(self, mod, name):
        f = C.c_void_p()
        self._check(self.cu.cuModuleGetFunction(C.byref(f), mod, name.encode()), f"cuModuleGetFunction({name})")
        return f

    def global_(self, mod, name):
        ptr, size = C.c_uint64(), C.c_size_t()
        self._check(self.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), mod, name.encode()),
                    f"cuModuleGetGlobal({name})")
        return ptr.value, size.value

    def write_constant(self, mod, name, data: bytes):
        """FractalRenderingModule.writeToConstantMemory: copies symbol-size bytes."""
        ptr, size = self.global_(mod, name)
        buf = C.create_string_buffer(bytes(data).ljust(size, b"\0"), max(size, len(data)))
        self._check(self.cu.cuMemcpyHtoD_v2(C.c_uint64(ptr), buf, C.c_size_t(size)), "cuMemcpyHtoD")
        return size

    def launch(self, fn, grid, block, params, sync=True):
        """params: list of ctypes objects; kernelParams[i] = &params[i] (Pointer.to(...) in JCuda).
        The launch goes to the legacy default stream, like JCuda's."""
        arr = (C.c_void_p * len(params))(*[C.cast(C.pointer(p), C.c_void_p) for p in params])
        self._check(self.cu.cuLaunchKernel(fn, grid[0], grid[1], 1, block[0], block[1], 1, 0, None, arr, None),
                    "cuLaunchKernel")
        if sync:
            self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


# Parameter arrays exactly as the Java kernels build them (CudaHelpers.pointerTo).
def main_params(out_ptr, pitch, w, h, rect, max_iter, max_ss, flags, double):
    R = C.c_double if double else C.c_float
    return [C.c_uint64(out_ptr), C.c_int64(pitch), (C.c_int32 * 2)(w, h), (R * 4)(*rect), C.c_int32(max_iter),
            C.c_float(max_ss), C.c_int32(flags)]


def advanced_params(out_ptr, pitch, w, h, rect, max_iter, max_ss, flags, rect_reused, in_ptr, in_pitch, focus,
                    double):
    R = C.c_double if double else C.c_float
    return main_params(out_ptr, pitch, w, h, rect, max_iter, max_ss, flags, double) + [
        (R * 4)(*rect_reused), C.c_uint64(in_ptr), C.c_int64(in_pitch), (C.c_int32 * 2)(*focus)]


def java_grid(w, h):
    """CudaFractalRenderer.launchRenderingKernel: 32x32 blocks, ceil(W/32) x ceil(H/32)."""
    return ((w + 31) // 32, (h + 31) // 32), (32, 32)
