"""The drop-in module files as the Java host uses them.

chaos-ultra's renderer loads a CUDA module per fractal by file path and
launches its kernels by name through JCuda (FractalRenderingModule.initialize,
J/cudarenderer/FractalRenderingModule.java:73-100; CudaFractalRenderer.
launchRenderingKernel, J/cudarenderer/CudaFractalRenderer.java:235-269).  This
module replays exactly those driver calls through ctypes -- cuModuleLoad,
cuModuleGetFunction, cuModuleGetGlobal + a host-to-device copy of the
symbol's size, cuLaunchKernel with a void** parameter array built in the
Java kernels' registration order -- so the modules under DROPIN_DIR /
DROPIN_PARITY_DIR (or any module with the same ABI) can be driven the way the
unchanged Java application drives them.  (J/ stands for
src/main/java/cz/cuni/mff/cgg/teichmaa/chaosultra/.)
"""
import ctypes as C

import numpy as np

# pixel_info_t, src/main/cuda/helpers.cuh:106-130: 16 bytes per record.
PIXEL_DTYPE = np.dtype([("value", "<f4"), ("weight", "<f4"), ("is_reused", "u1"), ("pad", "u1", 3),
                        ("weight_of_new_samples", "<f4")])
assert PIXEL_DTYPE.itemsize == 16

# The seven kernels FractalRenderingModule.initialize resolves
# (J/cudarenderer/FractalRenderingModule.java:91-97).
MODULE_KERNELS = ["fractalRenderMainFloat", "fractalRenderMainDouble", "fractalRenderAdvancedFloat",
                  "fractalRenderAdvancedDouble", "fractalRenderUnderSampled", "compose", "debug"]


def pitched(torch, w, h, pitch_align=512, device="cuda:0"):
    """A pitched w x h buffer of 16-byte records, like cuMemAllocPitch(w*16, h, 16)
    (DeviceMemoryDoubleBuffer2D.reallocate); returns (uint8 tensor, pitch)."""
    pitch = ((16 * w + pitch_align - 1) // pitch_align) * pitch_align
    buf = torch.zeros((h, pitch), dtype=torch.uint8, device=device)
    return buf, pitch


def read_pixels(buf, w):
    """Device pitched buffer -> (h, w) numpy array of pixel records."""
    host = buf.cpu().numpy()
    return np.ascontiguousarray(host[:, : 16 * w]).view(PIXEL_DTYPE).reshape(host.shape[0], w)


def same_pixels(a, b):
    """Field-wise comparison of two pixel arrays (padding bytes ignored);
    returns the mask of records that differ in any field, bit for bit."""
    m = np.zeros(a.shape, dtype=bool)
    for f in ("value", "weight", "is_reused", "weight_of_new_samples"):
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            m |= x.view(np.uint32) != y.view(np.uint32)
        else:
            m |= x != y
    return m


class Driver:
    """The CUDA driver calls JCuda makes for the Java host, through ctypes."""

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

    def read(self, ptr, nbytes):
        """Copy nbytes of device memory at ptr to a new bytes object (cuMemcpyDtoH)."""
        buf = C.create_string_buffer(nbytes)
        self._check(self.cu.cuMemcpyDtoH_v2(buf, C.c_uint64(ptr), C.c_size_t(nbytes)), "cuMemcpyDtoH")
        return buf.raw

    def read_pixels(self, ptr, pitch, w, h):
        """A pitched w x h array of pixel records at device address ptr -> (h, w) numpy array."""
        raw = np.frombuffer(self.read(ptr, pitch * h), dtype=np.uint8).reshape(h, pitch)
        return np.ascontiguousarray(raw[:, : 16 * w]).view(PIXEL_DTYPE).reshape(h, w)

    def launch(self, fn, grid, block, params, sync=True):
        """params: list of ctypes objects; kernelParams[i] = &params[i] (Pointer.to(...) in JCuda).
        The launch goes to the legacy default stream, like JCuda's."""
        arr = (C.c_void_p * len(params))(*[C.cast(C.pointer(p), C.c_void_p) for p in params])
        self._check(self.cu.cuLaunchKernel(fn, grid[0], grid[1], 1, block[0], block[1], 1, 0, None, arr, None),
                    "cuLaunchKernel")
        if sync:
            self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


# Parameter arrays exactly as the Java kernels build them (CudaHelpers.pointerTo;
# J/cudarenderer/KernelMain.java:19-20, KernelAdvanced.java:26-29).
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
