"""Helpers for the GPU tests: pitched device buffers (torch) and the replay of
the Java host's JCuda calls, from chaos_gb300.dropin, plus an upload helper."""
import numpy as np

from chaos_gb300.dropin import (MODULE_KERNELS, PIXEL_DTYPE, Driver, advanced_params, java_grid,  # noqa: F401
                                main_params, pitched, read_pixels, same_pixels)
from oracle.oracle import PIXEL_DTYPE as ORACLE_PIXEL_DTYPE

assert ORACLE_PIXEL_DTYPE == PIXEL_DTYPE


def upload_pixels(torch, arr, pitch_align=512):
    h, w = arr.shape
    buf, pitch = pitched(torch, w, h, pitch_align)
    host = np.zeros((h, pitch), dtype=np.uint8)
    host[:, : 16 * w] = np.ascontiguousarray(arr).view(np.uint8).reshape(h, 16 * w)
    buf.copy_(torch.from_numpy(host))
    return buf, pitch
