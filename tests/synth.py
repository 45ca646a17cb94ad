"""Seeded synthetic imaging-FCS stacks for CPU tests (numpy).

A 2D Brownian-motion model in the spirit of the reference simulator
(Imaging_FCS_1_52.java:13854-14409): particles diffuse on a periodic square,
each pixel receives the PSF-integrated emission rate (Gaussian PSF given by
its 1/e^2 radius), photon counts are Poisson, a camera offset is added, and an
optional single- or double-exponential bleach scales the rate
((1 - frac2) e^{-t/tau_bleach} + frac2 e^{-t/tau_bleach2}).  Output is uint16
[frames][height][width].
"""
import numpy as np
from scipy.special import erf


def brownian_stack(width=21, height=21, frames=20000, dt=1e-3, pixel=0.24, psf_w=0.4,
                   density=0.56, d=1.0, cps=10000.0, offset=100, tau_bleach=0.0, margin=2.0,
                   seed=1, d_map=None, tau_bleach2=0.0, frac2=0.0):
    rng = np.random.default_rng(seed)
    lx, ly = width * pixel + 2 * margin, height * pixel + 2 * margin
    n = max(1, int(round(density * lx * ly)))
    pos = np.column_stack([rng.uniform(0, lx, n), rng.uniform(0, ly, n)])
    if d_map is None:
        dpart = np.full(n, d)
    else:
        dpart = np.asarray(d_map(pos[:, 0] - margin, pos[:, 1] - margin), float)
    sig = psf_w / 2.0
    ex = np.arange(width + 1) * pixel + margin
    ey = np.arange(height + 1) * pixel + margin
    out = np.empty((frames, height, width), np.uint16)
    for t in range(frames):
        pos += rng.normal(0, 1, (n, 2)) * np.sqrt(2 * dpart * dt)[:, None]
        pos[:, 0] %= lx
        pos[:, 1] %= ly
        cx = 0.5 * (erf((ex[None, :] - pos[:, :1]) / (np.sqrt(2) * sig)))
        cy = 0.5 * (erf((ey[None, :] - pos[:, 1:]) / (np.sqrt(2) * sig)))
        px = np.diff(cx, axis=1)
        py = np.diff(cy, axis=1)
        rate = cps * dt * np.einsum("ny,nx->yx", py, px)
        if tau_bleach > 0 and tau_bleach2 > 0:
            rate *= (1 - frac2) * np.exp(-t * dt / tau_bleach) + frac2 * np.exp(-t * dt / tau_bleach2)
        elif tau_bleach > 0:
            rate *= np.exp(-t * dt / tau_bleach)
        out[t] = np.minimum(rng.poisson(rate) + offset, 65535)
    return out


def bleach_stack(width=8, height=8, frames=4000, amp=2000.0, tau1=0.4, tau2=4.0, frac2=0.6, dt=1e-3,
                 corr_frames=20.0, fluct=0.2, offset=100, seed=1):
    """Bright stack with a two-rate bleach and correlated intensity
    fluctuations: counts ~ Poisson(amp_pix b(t) (1 + fluct z(t))) + offset,
    b(t) = (1 - frac2) e^{-t/tau1} + frac2 e^{-t/tau2} (frac2 = 0: single
    rate), z an AR(1) process of unit variance and correlation time
    corr_frames per pixel.  The bleach curve dominates the trace, so
    exponential bleach fits have a unique least-squares minimum."""
    rng = np.random.default_rng(seed)
    t = np.arange(frames) * dt
    b = (1 - frac2) * np.exp(-t / tau1) + (frac2 * np.exp(-t / tau2) if frac2 > 0 else 0.0)
    rho = np.exp(-1.0 / corr_frames)
    z = np.empty((frames, height, width))
    z[0] = rng.normal(0, 1, (height, width))
    eps = rng.normal(0, np.sqrt(1 - rho * rho), (frames, height, width))
    for i in range(1, frames):
        z[i] = rho * z[i - 1] + eps[i]
    a = amp * rng.uniform(0.7, 1.3, (height, width))
    rate = a[None] * b[:, None, None] * np.clip(1 + fluct * z, 0, None)
    return np.minimum(rng.poisson(rate) + offset, 65535).astype(np.uint16)


# ----------------------------------------------------------------------------
# Host simulator in C (synth_host.c): the same Brownian model, fast enough for
# benchmark-sized stacks (128 x 128 x 50,000 in seconds on a many-core host),
# deterministic for a seed whatever the thread count.
# ----------------------------------------------------------------------------
import ctypes as _C
import os as _os
import subprocess as _sp

_HERE = _os.path.dirname(_os.path.abspath(__file__))
_SYNTH_LIB = _os.path.join(_HERE, "_build", "libsynth_host.so")
_synth = None


def build_host_synth(force: bool = False) -> str:
    src = _os.path.join(_HERE, "synth_host.c")
    if force or not _os.path.exists(_SYNTH_LIB) or _os.path.getmtime(_SYNTH_LIB) < _os.path.getmtime(src):
        _os.makedirs(_os.path.dirname(_SYNTH_LIB), exist_ok=True)
        _sp.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-fopenmp", "-shared", "-o", _SYNTH_LIB, src, "-lm"])
    return _SYNTH_LIB


def _synth_lib():
    global _synth
    if _synth is None:
        build_host_synth()
        _synth = _C.CDLL(_SYNTH_LIB)
        _synth.synth_brownian.restype = _C.c_int
        d, i = _C.c_double, _C.c_int
        _synth.synth_brownian.argtypes = [i, i, i, d, i, d, d, d, d, d, d, d, d, i, d, _C.c_uint64,
                                          _C.c_void_p, _C.c_void_p]
    return _synth


def host_stack(width, height, frames, *, frametime=1e-3, steps_per_frame=10, pixel_um=0.24, psf_um=0.4,
               density=500 / 900.0, d1=1.0, d2=0.0, fraction2=0.0, cps=10000.0, tau_bleach=0.0,
               offset=100, margin=2.0, seed=1, d_tile_map=None):
    """uint16 [frames][height][width] from the C host simulator."""
    out = np.empty((frames, height, width), np.uint16)
    dmap = None if d_tile_map is None else np.ascontiguousarray(d_tile_map, np.float32)
    rc = _synth_lib().synth_brownian(width, height, frames, frametime, steps_per_frame, pixel_um, psf_um,
                                     density, d1, d2, fraction2, cps, tau_bleach, offset, margin, seed,
                                     None if dmap is None else dmap.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise RuntimeError("synth_brownian failed")
    return out


def bench_stack(width=128, height=128, frames=50000, seed=1):
    """The plain-method-at-scale workload: D per 16 x 16 tile from
    U(0.2, 5) um^2/s, single-exponential bleach tau = 20 s, 500 particles per
    30 x 30 um, PSF 1/e^2 radius 0.4 um, 10,000 photons/s, offset 100."""
    rng = np.random.default_rng(seed)
    dmap = rng.uniform(0.2, 5.0, ((height + 15) // 16, (width + 15) // 16)).astype(np.float32)
    return host_stack(width, height, frames, tau_bleach=20.0, seed=seed, d_tile_map=dmap)
