"""Stack ingest and background-file statistics over the C ABI.

TiffStack reads uncompressed 16-bit TIFF stacks (imfcs_tiff_*: either byte
order, one IFD per frame or ImageJ's single-IFD stacks) into host arrays or
straight into CUDA tensors; background_stats computes loadBGRFile's
statistics (Imaging_FCS_1_52.java:6988-7103) of a device-resident background
stack (imfcs_background_stats).  Images are [height][width].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


class TiffStack:
    def __init__(self, path: str):
        self._L = _lib.load()
        h = C.c_void_p()
        w, hh, f = C.c_int(), C.c_int(), C.c_int()
        check(self._L.imfcs_tiff_open(str(path).encode(), C.byref(h), C.byref(w), C.byref(hh), C.byref(f)),
              "imfcs_tiff_open")
        self._h = h
        self.width, self.height, self.frames = int(w.value), int(hh.value), int(f.value)

    def close(self):
        if getattr(self, "_h", None):
            self._L.imfcs_tiff_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _range(self, first, count):
        if count is None:
            count = self.frames - first
        return int(first), int(count)

    def read(self, first: int = 0, count: int | None = None) -> np.ndarray:
        """Frames [first, first + count) as uint16 [count][height][width]."""
        first, count = self._range(first, count)
        out = np.empty((count, self.height, self.width), np.uint16)
        check(self._L.imfcs_tiff_read(self._h, first, count, C.c_void_p(out.ctypes.data)), "imfcs_tiff_read")
        return out

    def read_device(self, first: int = 0, count: int | None = None, out=None, stream=None):
        """Frames into a CUDA uint16 tensor (ordered on `stream`)."""
        import torch
        first, count = self._range(first, count)
        if out is None:
            out = torch.empty((count, self.height, self.width), dtype=torch.uint16, device="cuda")
        assert out.is_cuda and out.is_contiguous() and out.numel() == count * self.height * self.width
        s = stream if stream is not None else torch.cuda.current_stream()
        check(self._L.imfcs_tiff_read_device(self._h, first, count, C.c_void_p(out.data_ptr()),
                                             C.c_void_p(s.cuda_stream)), "imfcs_tiff_read_device")
        return out


def background_stats(dev_stack, stream=None) -> dict:
    """loadBGRFile's statistics of a CUDA uint16 stack [frames][height][width]:
    mean, var, covar [height][width], row_mean [height], col_mean [width]."""
    import torch
    assert dev_stack.is_cuda and dev_stack.is_contiguous() and dev_stack.dim() == 3
    f, h, w = dev_stack.shape
    out = {k: torch.empty(shape, dtype=torch.float64, device=dev_stack.device)
           for k, shape in (("mean", (h, w)), ("var", (h, w)), ("covar", (h, w)), ("row_mean", (h,)),
                            ("col_mean", (w,)))}
    s = stream if stream is not None else torch.cuda.current_stream()
    L = _lib.load()
    check(L.imfcs_background_stats(C.c_void_p(dev_stack.data_ptr()), w, h, f,
                                   *[C.c_void_p(out[k].data_ptr()) for k in ("mean", "var", "covar", "row_mean",
                                                                           "col_mean")],
                                   C.c_void_p(s.cuda_stream)), "imfcs_background_stats")
    s.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}
