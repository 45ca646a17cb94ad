"""The FCS_3p correlation model on the host (Imaging_FCS_1_52.java:13131-13408),
vectorised over pixels and lag times: the curve the plugin stores as a
pixel's fit function after a fit (java:10386 OLS, 10703 GLS) and writes to
the "Fit functions" sheets of its results workbook.

Parameters (SI): N, D, vx, vy, G, F2, D2, F3, D3, Ftrip, Ttrip.  Constants
(SI): ax, ay, s, sz, rx, ry, fitobsvol, q2, q3 -- the pixel size of the
binned window, the PSF 1/e^2 radius and axial size, the cross-correlation
displacement, the observation-area normalisation and the brightness ratios
of components 2 and 3.

G(tau) = (sum_k q_k^2 F_k L_k(tau) P_k(tau)) / (Z^2 N) * (1 + Ft/(1-Ft)
e^(-tau/Tt)) + G_inf, with F_1 = 1 - F2 - F3, q_1 = 1, Z = sum_k q_k F_k,
L_k the product over x and y of the overlap of two square pixels of side a
displaced by r under Gaussian spreading of width p0 = sqrt(4 D_k tau + s^2)
with flow v (normalised by 4 a_x^2 a_y^2 / fitobsvol), and P_k = (1 + 4
D_k tau / sz^2)^(-1/2) the axial (SPIM) factor (sz = infinity: TIRF)."""
from __future__ import annotations

import numpy as np
from scipy.special import erf

# The plugin's value of pi (java:13134).
_PI = 3.14159265359
_SQRT_PI = np.sqrt(_PI)


def _overlap_1d(a, r, v, tau, p0):
    """Overlap of two pixel windows of side a, centres r apart, along one
    axis, after spreading of width p0 and drift v * tau."""
    d1 = a + r - v * tau
    d2 = a - r + v * tau
    d3 = r - v * tau
    g = np.exp(-(d1 / p0) ** 2) + np.exp(-(d2 / p0) ** 2) - 2.0 * np.exp(-(d3 / p0) ** 2)
    return p0 / _SQRT_PI * g + d1 * erf(d1 / p0) + d2 * erf(d2 / p0) - 2.0 * d3 * erf(d3 / p0)


def _component(d, vx, vy, tau, cst):
    ax, ay, s, sz, rx, ry, obs = cst[:7]
    p0 = np.sqrt(4.0 * d * tau + s * s)
    lateral = _overlap_1d(ax, rx, vx, tau, p0) * _overlap_1d(ay, ry, vy, tau, p0) / (4.0 * (ax * ay) ** 2 / obs)
    axial = 1.0 / np.sqrt(1.0 + 4.0 * d * tau / (sz * sz))
    return lateral * axial


def fcs_model(par, cst, tau) -> np.ndarray:
    """G at lag times tau for parameters par: par [..., 11] (SI), cst [9],
    tau [T] -> [..., T]."""
    par = np.asarray(par, float)
    cst = np.asarray(cst, float)
    tau = np.asarray(tau, float)
    p = par[..., :, None]                      # broadcast the parameters over the lag axis
    n, d1, vx, vy, g = p[..., 0, :], p[..., 1, :], p[..., 2, :], p[..., 3, :], p[..., 4, :]
    f2, d2, f3, d3, ft, tt = p[..., 5, :], p[..., 6, :], p[..., 7, :], p[..., 8, :], p[..., 9, :], p[..., 10, :]
    q2, q3 = cst[7], cst[8]
    f1 = 1.0 - f2 - f3
    s = (f1 * _component(d1, vx, vy, tau, cst) + q2 * q2 * f2 * _component(d2, vx, vy, tau, cst) +
         q3 * q3 * f3 * _component(d3, vx, vy, tau, cst))
    z = f1 + q2 * f2 + q3 * f3
    # IEEE arithmetic as in the plugin: Ttrip = 0 gives exp(-inf) = 0 at
    # tau > 0 and NaN at tau = 0 (only a GLS fit function evaluates lag 0)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        trip = 1.0 + ft / (1.0 - ft) * np.exp(-tau / tt)
        return s / (z * z) / n * trip + g


def fit_curves(acf, fitres, fitted, cst, lagtime, *, var=None, covmats=None, gls=False, fitstart=1,
               fitend=None):
    """The plugin's per-pixel fit function and residuals after a fit
    (java:10383-10397 OLS, 10701-10710 GLS): for a fitted pixel the model at
    every lag of the fit (OLS: fitstart..fitend; GLS: every lag) and 0
    elsewhere; residuals weighted as the fit saw them -- OLS (acf - fit)/sd
    over the fit range, GLS L^-1 (acf - fit) over lags 1.. with L the
    Cholesky factor of the regularised covariance, acf - fit at lag 0.
    Pixels without a fit get 0 everywhere, as the plugin's failed fits.
    acf [n, ch]; fitres [n, 11]; fitted [n]; var [n, ch] (OLS); covmats
    [n, ch-1, ch-1] (GLS).  Returns (fit [n, ch], res [n, ch])."""
    acf = np.asarray(acf, float)
    n, ch = acf.shape
    fe = ch - 1 if fitend is None else int(fitend)
    fs = int(fitstart)
    fit = np.zeros((n, ch))
    res = np.zeros((n, ch))
    ok = np.asarray(fitted).astype(bool) & np.isfinite(np.asarray(fitres, float)).all(axis=1)
    if not ok.any():
        return fit, res
    model = fcs_model(np.asarray(fitres, float)[ok], cst, lagtime)
    if not gls:
        sel = slice(fs, fe + 1)
        fit[ok, sel] = model[:, sel]
        sd = np.sqrt(np.asarray(var, float)[ok, sel])
        res[ok, sel] = (acf[ok, sel] - model[:, sel]) / sd
        return fit, res
    fit[ok] = model
    res[ok, 0] = acf[ok, 0] - model[:, 0]
    cov = np.asarray(covmats, float).reshape(n, ch - 1, ch - 1)
    for j, pix in enumerate(np.flatnonzero(ok)):
        try:
            low = np.linalg.cholesky(cov[pix])
        except np.linalg.LinAlgError:
            continue
        res[pix, 1:] = np.linalg.solve(low, acf[pix, 1:] - model[j, 1:])
    return fit, res
