"""Whole-path API over the CUDA library: uint16 stack -> ACF, blocked
variance, fits, Bayes probabilities, diffusion law.

Device work runs on torch tensors (torch provides device memory and streams;
the compute is the library's CUDA kernels).  Host work takes numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import NCONST, NPARAM, check

# Plugin defaults (Imaging_FCS_1_52.java:185-205, 1958-1970): N=1, D=1 um^2/s,
# G=0, everything else 0; N, D, G free.
DEFAULT_INIT = (1.0, 1e-12, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
DEFAULT_FREE = (1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0)


def obsvol_2d(ax: float, ay: float, s: float) -> float:
    """Observation area normalisation obsvolFCS_ST2D1p(2) (java:13670-13702), SI."""
    sqrpi = math.sqrt(3.14159265359)
    px = s / sqrpi * (2 * math.exp(-(ax / s) ** 2) - 2) + 2 * ax * math.erf(ax / s)
    py = s / sqrpi * (2 * math.exp(-(ay / s) ** 2) - 2) + 2 * ay * math.erf(ay / s)
    return 4 * (ax * ay) ** 2 / (px * py)


def model_constants(pixel_um: float = 0.24, binx: int = 1, biny: int = 1, psf_um: float = 0.4,
                    sz_um: float = 1e6 * 0.515 / 1.49, cfx: int = 0, cfy: int = 0,
                    q2: float = 1.0, q3: float = 1.0) -> np.ndarray:
    """FCS_3p constants (java:13135-13145, prepareFit 10028-10038) in SI units:
    ax, ay, s, sz, rx, ry, fitobsvol, q2, q3.  psf_um is the 1/e^2 radius."""
    ax = pixel_um * 1e-6 * binx
    ay = pixel_um * 1e-6 * biny
    s = psf_um * 1e-6
    rx = ax * cfx / binx
    ry = ay * cfy / biny
    return np.array([ax, ay, s, sz_um * 1e-6, rx, ry, obsvol_2d(ax, ay, s), q2, q3], dtype=float)


@dataclass
class FCSConfig:
    width: int
    height: int
    frames: int
    first: int = 0
    num: int | None = None
    out_w: int | None = None
    out_h: int | None = None
    map_x0: int = 0
    map_y0: int = 0
    binx: int = 1
    biny: int = 1
    pixbinx: int | None = None
    pixbiny: int | None = None
    cfx: int = 0
    cfy: int = 0
    background: int = 0
    p: int = 16
    q: int = 8
    frametime: float = 1e-3
    bleach: int = _lib.BLEACH_NONE
    poly_order: int = 4
    gls: bool = False
    bayes: bool = False
    do_fit: bool = True
    fitstart: int = 1
    fitend: int | None = None
    max_iter: int = 2000
    init: tuple = DEFAULT_INIT
    free_mask: tuple = DEFAULT_FREE
    cst: np.ndarray = field(default_factory=model_constants)

    def __post_init__(self):
        if self.num is None:
            self.num = self.frames - self.first
        if self.pixbinx is None:
            self.pixbinx = self.binx
        if self.pixbiny is None:
            self.pixbiny = self.biny
        if self.out_w is None:
            self.out_w = (self.width - max(0, self.cfx) - self.binx) // self.pixbinx + 1
        if self.out_h is None:
            self.out_h = (self.height - max(0, self.cfy) - self.biny) // self.pixbiny + 1

    @property
    def chanum(self) -> int:
        return int(self.p + (self.q - 1) * self.p / 2 + 1)

    @property
    def npix(self) -> int:
        return self.out_w * self.out_h

    def to_c(self) -> _lib.Config:
        c = _lib.Config()
        for name in ("width", "height", "frames", "first", "num", "out_w", "out_h", "map_x0", "map_y0",
                     "binx", "biny", "pixbinx", "pixbiny", "cfx", "cfy", "background", "p", "q",
                     "bleach", "poly_order", "max_iter", "fitstart"):
            setattr(c, name, int(getattr(self, name)))
        c.frametime = float(self.frametime)
        c.gls, c.bayes, c.do_fit = int(self.gls), int(self.bayes), int(self.do_fit)
        c.fitend = int(self.chanum - 1 if self.fitend is None else self.fitend)
        for i in range(NPARAM):
            c.init[i] = float(self.init[i])
            c.free_mask[i] = int(self.free_mask[i])
        for i in range(NCONST):
            c.cst[i] = float(self.cst[i])
        return c


_OUT_SPEC = {  # name -> (dtype, per-pixel shape (function of chanum))
    "acf": ("f8", lambda c: (c,)), "var": ("f8", lambda c: (c,)), "sd": ("f8", lambda c: (c,)),
    "blocked_ind": ("i4", lambda c: ()), "blocked_ok": ("i4", lambda c: ()),
    "nb_mean": ("f8", lambda c: ()), "nb_cov": ("f8", lambda c: ()),
    "fitres": ("f4", lambda c: (NPARAM,)), "chi2": ("f4", lambda c: ()), "fitted": ("i4", lambda c: ()),
    "iterations": ("i4", lambda c: ()), "bayes_prob": ("f4", lambda c: (2,)),
    "covmats": ("f8", lambda c: (c - 1, c - 1)),
}


def output_names(cfg: FCSConfig) -> list[str]:
    names = ["acf", "var", "sd", "blocked_ind", "blocked_ok", "nb_mean", "nb_cov"]
    if cfg.do_fit:
        names += ["fitres", "chi2", "fitted", "iterations"]
    if cfg.bayes:
        names += ["bayes_prob"]
    if cfg.gls:
        names += ["covmats"]
    return names


def _outputs_struct(ptrs: dict) -> _lib.Outputs:
    o = _lib.Outputs()
    for k, v in ptrs.items():
        setattr(o, k, v)
    return o


class Plan:
    """A device plan for one configuration (imfcs_plan_*)."""

    def __init__(self, cfg: FCSConfig):
        self.cfg = cfg
        self._L = _lib.load()
        self._c = cfg.to_c()
        h = C.c_void_p()
        check(self._L.imfcs_plan_create(C.byref(self._c), C.byref(h)), "imfcs_plan_create")
        self._h = h

    @property
    def scratch_bytes(self) -> int:
        return int(self._L.imfcs_plan_scratch_bytes(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._L.imfcs_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    STAGES = ("trace+bleach", "stream", "blocking", "correlator", "gls", "fits")

    def set_timing(self, enable: bool = True):
        check(self._L.imfcs_plan_set_timing(self._h, int(enable)), "imfcs_plan_set_timing")

    def stage_times(self) -> dict:
        """Per-stage device times (ms) of the last execution (after a sync)."""
        ms = (C.c_float * len(self.STAGES))()
        n = self._L.imfcs_plan_stage_times(self._h, ms, len(self.STAGES))
        if n < 0:
            raise _lib.ImfcsError(_lib.last_error())
        return {k: float(ms[i]) for i, k in enumerate(self.STAGES)}

    def kernel_launches(self) -> int:
        """CUDA kernels launched by the last execution."""
        n = self._L.imfcs_plan_kernel_launches(self._h)
        if n < 0:
            raise _lib.ImfcsError(_lib.last_error())
        return int(n)

    def bleach_params(self) -> np.ndarray:
        """Per-trace bleach parameters of the last execution (diagnostic)."""
        n = self.cfg.npix * (2 if (self.cfg.cfx or self.cfg.cfy) else 1)
        out = np.zeros((n, 16), np.float32)
        got = self._L.imfcs_plan_bleach_params(self._h, C.c_void_p(out.ctypes.data), n)
        if got < 0:
            raise _lib.ImfcsError(_lib.last_error())
        return out

    def set_background_image(self, bg):
        """Per-pixel background (imfcs_plan_set_background_image): bg
        [height][width] of the input frames, the mean background of each raw
        pixel (rounded per pixel as the plugin does); None = the scalar one."""
        if bg is None:
            check(self._L.imfcs_plan_set_background_image(self._h, None), "imfcs_plan_set_background_image")
            return
        a = np.ascontiguousarray(bg, np.float64)
        if a.shape != (self.cfg.height, self.cfg.width):
            raise ValueError(f"background image must be {self.cfg.height} x {self.cfg.width}")
        check(self._L.imfcs_plan_set_background_image(self._h, C.c_void_p(a.ctypes.data)),
              "imfcs_plan_set_background_image")

    def set_surrogate(self, surrogate, mode: int = 1):
        """Seed the do_fit LM from a trained surrogate (imfcs_plan_set_surrogate):
        mode 1 refits failed seeded fits from the configured initial values;
        mode 2 also runs plain LM on every pixel and keeps the plain result
        where the seeded chi^2 is more than 1 % higher; None / 0 detaches."""
        h = None if surrogate is None else surrogate.handle
        check(self._L.imfcs_plan_set_surrogate(self._h, h, int(mode if surrogate is not None else 0)),
              "imfcs_plan_set_surrogate")
        self._surrogate = surrogate   # keep the handle alive while attached

    def surrogate_stats(self) -> dict:
        """Refit counts of the last seeded execution (synchronises)."""
        a, b = C.c_int(), C.c_int()
        check(self._L.imfcs_plan_surrogate_stats(self._h, C.byref(a), C.byref(b)), "imfcs_plan_surrogate_stats")
        return {"refit": int(a.value), "worse_than_plain": int(b.value)}

    def alloc_device_outputs(self, device="cuda"):
        import torch
        tmap = {"f8": torch.float64, "f4": torch.float32, "i4": torch.int32}
        out = {}
        for n in output_names(self.cfg):
            dt, shp = _OUT_SPEC[n]
            out[n] = torch.empty((self.cfg.npix, *shp(self.cfg.chanum)), dtype=tmap[dt], device=device)
        return out

    def execute(self, stack, outputs: dict, stream=None):
        """stack: CUDA uint16 tensor [frames][height][width]; outputs: CUDA
        tensors from alloc_device_outputs.  Asynchronous on `stream`."""
        import torch
        assert stack.is_cuda and stack.is_contiguous()
        s = stream if stream is not None else torch.cuda.current_stream()
        o = _outputs_struct({k: v.data_ptr() for k, v in outputs.items()})
        check(self._L.imfcs_plan_execute(self._h, C.c_void_p(stack.data_ptr()), C.byref(o),
                                         C.c_void_p(s.cuda_stream)), "imfcs_plan_execute")
        return outputs

    def execute_host(self, stack: np.ndarray, outputs: dict | None = None, stream=None) -> dict:
        """Host stack in, host results out (copies inside the call)."""
        stack = np.ascontiguousarray(stack, dtype=np.uint16)
        if outputs is None:
            outputs = {}
            for n in output_names(self.cfg):
                dt, shp = _OUT_SPEC[n]
                outputs[n] = np.empty((self.cfg.npix, *shp(self.cfg.chanum)), dtype=dt)
        o = _outputs_struct({k: v.ctypes.data for k, v in outputs.items()})
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        check(self._L.imfcs_plan_execute_host(self._h, C.c_void_p(stack.ctypes.data), C.byref(o), sp),
              "imfcs_plan_execute_host")
        return outputs

    def execute_host_async(self, stack: np.ndarray, outputs: dict, stream=None):
        """Enqueue one host-buffer execution (imfcs_plan_execute_host_async):
        the copy of the next stack overlaps this one's execution.  Use
        page-locked arrays for stack and outputs; results are valid after
        synchronize()."""
        assert stack.flags["C_CONTIGUOUS"] and stack.dtype == np.uint16
        self._async_keep = (stack, outputs)          # alive until synchronised
        o = _outputs_struct({k: v.ctypes.data for k, v in outputs.items()})
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        check(self._L.imfcs_plan_execute_host_async(self._h, C.c_void_p(stack.ctypes.data), C.byref(o), sp),
              "imfcs_plan_execute_host_async")

    def synchronize(self, stream=None):
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        check(self._L.imfcs_plan_synchronize(self._h, sp), "imfcs_plan_synchronize")

    def set_corr_tile(self, cta: int, seg_extra: int, tail_extra: int | None = None):
        """Correlator tile of the level chain: cta pixels per CTA (32 or 64),
        the pair kernels' frame segments 2^seg_extra and the tail kernel's
        2^tail_extra (default: seg_extra) times the shortest legal one."""
        t = seg_extra if tail_extra is None else tail_extra
        check(self._L.imfcs_plan_set_corr_tile(self._h, int(cta), int(seg_extra), int(t)),
              "imfcs_plan_set_corr_tile")

    def corr_tile(self) -> tuple[int, int, int]:
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(self._L.imfcs_plan_get_corr_tile(self._h, C.byref(a), C.byref(b), C.byref(c)),
              "imfcs_plan_get_corr_tile")
        return int(a.value), int(b.value), int(c.value)

    def autotune(self, stack, outputs: dict, stream=None) -> list[dict]:
        """Time the correlator at every tile on this stack, keep the fastest
        (imfcs_plan_autotune); returns the trials."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        o = _outputs_struct({k: v.data_ptr() for k, v in outputs.items()})
        trials = (_lib.CorrTile * 16)()
        n = C.c_int()
        check(self._L.imfcs_plan_autotune(self._h, C.c_void_p(stack.data_ptr()), C.byref(o),
                                          C.c_void_p(s.cuda_stream), trials, 16, C.byref(n)), "imfcs_plan_autotune")
        return [{"cta": t.cta, "seg_extra": t.seg_extra, "tail_extra": t.tail_extra, "ms": float(t.ms)}
                for t in trials[:n.value]]


def lag_tables(p: int, q: int) -> tuple[np.ndarray, np.ndarray]:
    """Lag (frames) and bin width of every channel (java:7391-7424): level 0
    lags 0..p, then p/2 lags per level k = 1..q-1 at bin width 2^k."""
    hb = p // 2
    ch = int(p + (q - 1) * p / 2 + 1)
    lag = np.zeros(ch, np.int64)
    samp = np.ones(ch)
    for x in range(hb + 1):
        lag[x] = x
    for x in range(1, q + 1):
        for y in range(1, hb + 1):
            i = x * hb + y
            if i < ch:
                lag[i] = 2 ** (x - 1) * y + (p // 4) * 2 ** x
                if x >= 2:
                    samp[i] = 2 ** (x - 1)
    return lag, samp


def batch_configs(width: int, height: int, frames: int, binnings=(1, 2, 3, 4, 5),
                  offsets=((0, 0), (1, 0), (2, 0), (0, 1), (1, 1), (2, 1), (0, 2), (1, 2), (2, 2)),
                  **kw) -> list[FCSConfig]:
    """One job per (binning, offset): non-overlapping binning (pixel step =
    binning, as the diffusion law's "All" mode), cross-correlation of each
    binned window with the window displaced by (dx, dy) input pixels
    ((0, 0): autocorrelation); every job fits N, D, G with the model
    constants of its binning."""
    cfgs = []
    psf = kw.pop("psf_um", 0.4)
    pixel = kw.pop("pixel_um", 0.24)
    for b in binnings:
        for dx, dy in offsets:
            cfgs.append(FCSConfig(width=width, height=height, frames=frames, binx=b, biny=b, cfx=dx, cfy=dy,
                                  cst=model_constants(pixel_um=pixel, binx=b, biny=b, psf_um=psf, cfx=dx, cfy=dy),
                                  **kw))
    return cfgs


class Batch:
    """Several jobs over one stack as one CUDA graph (imfcs_batch_*)."""

    def __init__(self, cfgs: list[FCSConfig], lanes: int = 1):
        self.cfgs = list(cfgs)
        self._L = _lib.load()
        arr = (_lib.Config * len(self.cfgs))(*[c.to_c() for c in self.cfgs])
        h = C.c_void_p()
        check(self._L.imfcs_batch_create(arr, len(self.cfgs), int(lanes), C.byref(h)), "imfcs_batch_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.imfcs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def lanes(self) -> int:
        return int(self._L.imfcs_batch_lanes(self._h))

    @property
    def scratch_bytes(self) -> int:
        return int(self._L.imfcs_batch_scratch_bytes(self._h))

    def kernel_launches(self) -> int:
        return int(self._L.imfcs_batch_kernel_launches(self._h))

    def job_info(self, i: int) -> dict:
        v = [C.c_int() for _ in range(6)]
        ms = C.c_float()
        check(self._L.imfcs_batch_job_info(self._h, i, *[C.byref(x) for x in v], C.byref(ms)),
              "imfcs_batch_job_info")
        return {"npix": v[0].value, "chanum": v[1].value, "lane": v[2].value, "cta": v[3].value,
                "seg_extra": v[4].value, "tail_extra": v[5].value, "ms": float(ms.value)}

    def alloc_device_outputs(self, device="cuda") -> list[dict]:
        import torch
        tmap = {"f8": torch.float64, "f4": torch.float32, "i4": torch.int32}
        outs = []
        for c in self.cfgs:
            o = {}
            for n in output_names(c):
                dt, shp = _OUT_SPEC[n]
                o[n] = torch.empty((c.npix, *shp(c.chanum)), dtype=tmap[dt], device=device)
            outs.append(o)
        return outs

    def _outs(self, outputs: list[dict]):
        arr = (_lib.Outputs * len(self.cfgs))()
        for i, o in enumerate(outputs):
            arr[i] = _outputs_struct({k: v.data_ptr() for k, v in o.items()})
        return arr

    def execute(self, stack, outputs: list[dict], stream=None):
        """stack: CUDA uint16 tensor [frames][height][width]; outputs: one
        dict of CUDA tensors per job.  Asynchronous on `stream`."""
        import torch
        assert stack.is_cuda and stack.is_contiguous()
        s = stream if stream is not None else torch.cuda.current_stream()
        check(self._L.imfcs_batch_execute(self._h, C.c_void_p(stack.data_ptr()), self._outs(outputs),
                                          C.c_void_p(s.cuda_stream)), "imfcs_batch_execute")
        return outputs

    def synchronize(self, stream=None):
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        check(self._L.imfcs_batch_synchronize(self._h, sp), "imfcs_batch_synchronize")

    def autotune(self, stack, outputs: list[dict], max_lanes: int = 4, stream=None) -> list[float]:
        """Tune the jobs' correlator tiles and the lane count on this stack
        (imfcs_batch_autotune); returns the graph time per lane count."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        ms = (C.c_float * max_lanes)()
        check(self._L.imfcs_batch_autotune(self._h, C.c_void_p(stack.data_ptr()), self._outs(outputs),
                                           C.c_void_p(s.cuda_stream), int(max_lanes), ms), "imfcs_batch_autotune")
        return [float(x) for x in ms]


def band_windows(cfg: FCSConfig, band_rows: int) -> list[dict]:
    """The band split imfcs_bands uses (imfcs_band_window; host arithmetic,
    no device): per band its first output row, the output rows it adds, the
    input row of its buffer's first row and its input rows."""
    L = _lib.load()
    c = cfg.to_c()
    v = [C.c_int() for _ in range(5)]
    n = L.imfcs_band_window(C.byref(c), int(band_rows), 0, *[C.byref(x) for x in v])
    if n < 0:
        raise _lib.ImfcsError(_lib.last_error())
    out = []
    for b in range(n):
        L.imfcs_band_window(C.byref(c), int(band_rows), b, *[C.byref(x) for x in v])
        out.append({"out_row0": v[0].value, "new_row0": v[1].value, "new_rows": v[2].value,
                    "in_row0": v[3].value, "in_rows": v[4].value})
    return out


class Bands:
    """Band-streamed execution of a host stack larger than the device memory
    granted (imfcs_bands_*): bands of output rows, each band's input rows
    copied while the previous band computes.  band_rows = 0 sizes the bands
    from max_device_bytes (0: 90 % of the free device memory)."""

    def __init__(self, cfg: FCSConfig, band_rows: int = 0, max_device_bytes: int = 0):
        self.cfg = cfg
        self._L = _lib.load()
        self._c = cfg.to_c()
        h = C.c_void_p()
        check(self._L.imfcs_bands_create(C.byref(self._c), int(band_rows), int(max_device_bytes), C.byref(h)),
              "imfcs_bands_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.imfcs_bands_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def geometry(self) -> dict:
        r, n, b = C.c_int(), C.c_int(), C.c_size_t()
        check(self._L.imfcs_bands_geometry(self._h, C.byref(r), C.byref(n), C.byref(b)), "imfcs_bands_geometry")
        return {"band_rows": r.value, "bands": n.value, "device_bytes": int(b.value)}

    def set_corr_tile(self, cta: int, seg_extra: int, tail_extra: int | None = None):
        t = seg_extra if tail_extra is None else tail_extra
        check(self._L.imfcs_plan_set_corr_tile(self._L.imfcs_bands_plan(self._h), int(cta), int(seg_extra), int(t)),
              "imfcs_plan_set_corr_tile")

    def set_background_image(self, bg):
        """Per-pixel background [height][width] of the whole input frame
        (imfcs_bands_set_background_image); None = the scalar one."""
        if bg is None:
            check(self._L.imfcs_bands_set_background_image(self._h, None), "imfcs_bands_set_background_image")
            return
        a = np.ascontiguousarray(bg, np.float64)
        if a.shape != (self.cfg.height, self.cfg.width):
            raise ValueError(f"background image must be {self.cfg.height} x {self.cfg.width}")
        check(self._L.imfcs_bands_set_background_image(self._h, C.c_void_p(a.ctypes.data)),
              "imfcs_bands_set_background_image")

    def execute_host(self, stack: np.ndarray, outputs: dict | None = None, stream=None) -> dict:
        """Host stack [frames][height][width] in, host results out."""
        stack = np.ascontiguousarray(stack, dtype=np.uint16)
        if stack.shape != (self.cfg.frames, self.cfg.height, self.cfg.width):
            raise ValueError(f"stack must be {self.cfg.frames} x {self.cfg.height} x {self.cfg.width}")
        if outputs is None:
            outputs = {}
            for n in output_names(self.cfg):
                dt, shp = _OUT_SPEC[n]
                outputs[n] = np.empty((self.cfg.npix, *shp(self.cfg.chanum)), dtype=dt)
        o = _outputs_struct({k: v.ctypes.data for k, v in outputs.items()})
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        check(self._L.imfcs_bands_execute(self._h, C.c_void_p(stack.ctypes.data), C.byref(o), sp),
              "imfcs_bands_execute")
        return outputs


def run_host(stack: np.ndarray, cfg: FCSConfig) -> dict:
    plan = Plan(cfg)
    try:
        return plan.execute_host(stack)
    finally:
        plan.close()


def simulate(width: int, height: int, frames: int, *, frametime: float = 1e-3,
             steps_per_frame: int = 10, pixel_um: float = 0.24, psf_um: float = 0.4,
             density: float = 500 / 900.0, d1: float = 1.0, d2: float = 0.0, fraction2: float = 0.0,
             cps: float = 10000.0, tau_bleach: float = 0.0, offset: int = 100,
             read_noise: float = 0.0, margin: float = 2.0, seed: int = 1, d_tile_map=None,
             device="cuda"):
    """GPU Monte-Carlo stack (imfcs_simulate) as a CUDA uint16 tensor."""
    import torch
    L = _lib.load()
    p = _lib.SimParams(width=width, height=height, frames=frames, frametime=frametime,
                       steps_per_frame=steps_per_frame, pixel_size=pixel_um, psf_radius=psf_um,
                       density=density, d1=d1, d2=d2, fraction2=fraction2, cps=cps,
                       tau_bleach=tau_bleach, offset=offset, read_noise=read_noise, margin=margin,
                       seed=seed)
    out = torch.empty((frames, height, width), dtype=torch.uint16, device=device)
    dmap = None
    if d_tile_map is not None:
        dmap = torch.as_tensor(np.ascontiguousarray(d_tile_map, np.float32), device=device)
    s = torch.cuda.current_stream()
    check(L.imfcs_simulate(C.byref(p), None if dmap is None else C.c_void_p(dmap.data_ptr()),
                           C.c_void_p(out.data_ptr()), C.c_void_p(s.cuda_stream)), "imfcs_simulate")
    return out


def to_numpy_u16(t) -> np.ndarray:
    import torch
    return t.view(torch.int16).cpu().numpy().view(np.uint16)
