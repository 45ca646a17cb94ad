"""Seeded synthetic imaging-FCS stacks for CPU tests (numpy).

A 2D Brownian-motion model in the spirit of the reference simulator
(Imaging_FCS_1_52.java:13854-14409): particles diffuse on a periodic square,
each pixel receives the PSF-integrated emission rate (Gaussian PSF given by
its 1/e^2 radius), photon counts are Poisson, a camera offset is added, and an
optional single-exponential bleach scales the rate.  Output is uint16
[frames][height][width].
"""
import numpy as np
from scipy.special import erf


def brownian_stack(width=21, height=21, frames=20000, dt=1e-3, pixel=0.24, psf_w=0.4,
                   density=0.56, d=1.0, cps=10000.0, offset=100, tau_bleach=0.0, margin=2.0,
                   seed=1, d_map=None):
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
        if tau_bleach > 0:
            rate *= np.exp(-t * dt / tau_bleach)
        out[t] = np.minimum(rng.poisson(rate) + offset, 65535)
    return out
