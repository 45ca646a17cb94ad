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
