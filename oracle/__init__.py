"""FP64 CPU oracle for the Imaging_FCS 1.52 correlation-and-fit path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline / reference arm as the checker.  The product package
(imaging_fcs_1_52_gb300) never imports it.

The C library (imfcs_oracle.c) restates the reference's Java CPU path
(Imaging_FCS_1_52.java); see its header for the lines each function follows
and for the parity status ("unpinned" beyond the documented lag example,
analytic cases and the MINPACK cross-check).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libimfcs_oracle.so")
_lib = None

NPARAM = 11
NCONST = 9
BLEACH_NONE, BLEACH_SINGLE_EXP, BLEACH_DOUBLE_EXP, BLEACH_POLY = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("imfcs_oracle.c", "imfcs_oracle.h")
    ):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags="C_CONTIGUOUS")


class Config(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("frames", C.c_int),
        ("first", C.c_int), ("num", C.c_int),
        ("out_w", C.c_int), ("out_h", C.c_int), ("map_x0", C.c_int), ("map_y0", C.c_int),
        ("binx", C.c_int), ("biny", C.c_int), ("pixbinx", C.c_int), ("pixbiny", C.c_int),
        ("cfx", C.c_int), ("cfy", C.c_int), ("background", C.c_int),
        ("p", C.c_int), ("q", C.c_int), ("frametime", C.c_double),
        ("bleach", C.c_int), ("poly_order", C.c_int),
        ("gls", C.c_int), ("bayes", C.c_int), ("do_fit", C.c_int),
        ("fitstart", C.c_int), ("fitend", C.c_int), ("max_iter", C.c_int),
        ("init", C.c_double * NPARAM), ("free_mask", C.c_int * NPARAM),
        ("cst", C.c_double * NCONST), ("threads", C.c_int),
    ]


def _declare(L):
    L.imfcs_o_chanum.restype = C.c_int
    L.imfcs_o_chanum.argtypes = [C.c_int, C.c_int]
    L.imfcs_o_lag_tables.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _dp, _dp]
    L.imfcs_o_get_intensity.argtypes = [_u16p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, _dp]
    L.imfcs_o_intensity_trace.argtypes = [_u16p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_void_p, C.c_int, C.c_double, _dp, _dp]
    L.imfcs_o_poly_fit.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp]
    L.imfcs_o_exp_fit.argtypes = [_dp, _dp, C.c_int, _dp]
    L.imfcs_o_dexp_fit.argtypes = [_dp, _dp, C.c_int, _dp]
    L.imfcs_o_exp_fit_rate.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp, _dp]
    L.imfcs_o_bleach_apply.argtypes = [_dp, C.c_int, C.c_double, C.c_int, C.c_int, _dp]
    L.imfcs_o_block_transform.restype = C.c_int
    L.imfcs_o_block_transform.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, _ip, _dp, _dp,
                                          C.c_double, C.POINTER(C.c_int), C.c_void_p]
    L.imfcs_o_calculate_cf.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, _ip, _dp,
                                       _dp, C.c_int, _dp, _dp, _dp, C.c_void_p]
    L.imfcs_o_fcs_model.argtypes = [_dp, _dp, C.c_double, C.POINTER(C.c_double), C.c_void_p]
    L.imfcs_o_obsvol.restype = C.c_double
    L.imfcs_o_obsvol.argtypes = [C.c_double, C.c_double, C.c_double]
    L.imfcs_o_fit_ols.restype = C.c_int
    L.imfcs_o_fit_ols.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp, _ip, _dp,
                                  C.c_int, _dp, C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.POINTER(C.c_int)]
    L.imfcs_o_fit_gls.restype = C.c_int
    L.imfcs_o_fit_gls.argtypes = [_dp, _dp, _dp, C.c_int, _dp, _ip, _dp, C.c_int, _dp,
                                  C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.POINTER(C.c_int)]
    L.imfcs_o_bayes.restype = C.c_int
    L.imfcs_o_bayes.argtypes = [_dp, _dp, C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, C.c_int,
                                _dp, _dp, C.c_int, _dp, _dp, _dp]
    L.imfcs_o_line_fit.restype = C.c_int
    L.imfcs_o_line_fit.argtypes = [_dp, _dp, _dp, C.c_int, _dp]
    L.imfcs_o_run.restype = C.c_int
    L.imfcs_o_run.argtypes = [C.POINTER(Config), _u16p, C.c_void_p, _dp, _dp, _dp, _ip, _ip,
                              _dp, _dp, _ip, C.c_void_p, C.c_void_p]


# ----------------------------------------------------------------------------- helpers
def chanum(p: int, q: int) -> int:
    return lib().imfcs_o_chanum(p, q)


def lag_tables(p: int, q: int, num: int):
    c = chanum(p, q)
    lag = np.zeros(c, np.int32)
    samp = np.zeros(c)
    mtab = np.zeros(c)
    lib().imfcs_o_lag_tables(p, q, num, lag, samp, mtab)
    return lag, samp, mtab


def get_intensity(stack, px, py, binx=1, biny=1, bckg=0, first=0, num=None, bgr=None):
    stack = np.ascontiguousarray(stack, np.uint16)
    t, h, w = stack.shape
    num = t - first if num is None else num
    out = np.zeros(num + 1)
    bgr_p = None if bgr is None else np.ascontiguousarray(bgr, np.int32).ctypes.data
    lib().imfcs_o_get_intensity(stack, w, h, first, num, px, py, binx, biny, bckg, bgr_p, out)
    return out


def intensity_trace(stack, px, py, binx=1, biny=1, bckg=0, frametime=1e-3, first=0, num=None,
                    bgr=None, bg_window=None):
    """Averaged trace of the window at (px, py); bg_window = (x, y) of the
    window whose background-image values are subtracted (default: its own)."""
    stack = np.ascontiguousarray(stack, np.uint16)
    t, h, w = stack.shape
    num = t - first if num is None else num
    nopit = min(num, 1000)
    tr = np.zeros(nopit)
    tt = np.zeros(nopit)
    bgr_p = None if bgr is None else np.ascontiguousarray(bgr, np.int32).ctypes.data
    bgx, bgy = (px, py) if bg_window is None else bg_window
    lib().imfcs_o_intensity_trace(stack, w, h, first, num, px, py, bgx, bgy, binx, biny, bckg, bgr_p, nopit,
                                  frametime, tr, tt)
    return tr, tt


def poly_fit(y, t, order):
    coef = np.zeros(order + 1)
    st = lib().imfcs_o_poly_fit(np.ascontiguousarray(y, float), np.ascontiguousarray(t, float),
                                len(y), order, coef)
    return coef, st


def exp_fit(y, t):
    res = np.zeros(3)
    st = lib().imfcs_o_exp_fit(np.ascontiguousarray(y, float), np.ascontiguousarray(t, float),
                               len(y), res)
    return res, st


def dexp_fit(y, t):
    res = np.zeros(5)
    st = lib().imfcs_o_dexp_fit(np.ascontiguousarray(y, float), np.ascontiguousarray(t, float),
                                len(y), res)
    return res, st


def exp_fit_rate(y, t, two=False):
    """Rate-form exponential fit (f0, s1, k1 [, s2, k2]) and standard errors."""
    k = 5 if two else 3
    rate, sig = np.zeros(k), np.zeros(k)
    st = lib().imfcs_o_exp_fit_rate(np.ascontiguousarray(y, float), np.ascontiguousarray(t, float), len(y),
                                    int(two), rate, sig)
    return rate, sig, st


def bleach_rate_determined(stack, out_w, out_h, *, binx=1, biny=1, cfx=0, cfy=0, background=0,
                           frametime=1e-3, two=False):
    """Per output pixel: True where every exponential bleach rate of its
    trace(s) is determined by the averaged trace (standard error below the
    rate's value).  Elsewhere the least-squares minimum is flat along a curve
    and the correction depends on where an optimiser stops."""
    out = np.ones(out_w * out_h, bool)
    for p in range(out_w * out_h):
        ox, oy = p % out_w, p // out_w
        for dx, dy in ((0, 0), (cfx, cfy)) if (cfx or cfy) else ((0, 0),):
            tr, tt = intensity_trace(stack, ox * binx + dx, oy * biny + dy, binx=binx, biny=biny,
                                     bckg=background, frametime=frametime)
            rate, sig, st = exp_fit_rate(tr, tt, two)
            ks = rate[2::2]
            if st != 0 or not np.all(sig[2::2] < np.abs(ks)):
                out[p] = False
    return out


def bleach_apply(intdat, frametime, mode, res, order=0):
    out = np.array(intdat, dtype=float, copy=True)
    lib().imfcs_o_bleach_apply(out, len(out) - 1, frametime, mode, order,
                               np.ascontiguousarray(res, float))
    return out


def block_transform(c0, c1, p, q, frametime=1e-3, want_curve=False):
    num = len(c0) - 1
    lag, samp, mtab = lag_tables(p, q, num)
    ok = C.c_int(0)
    blocknum = int(np.floor(np.log(mtab[1]) / np.log(2))) - 2
    curve = np.zeros(3 * blocknum)
    ind = lib().imfcs_o_block_transform(np.ascontiguousarray(c0, float),
                                        np.ascontiguousarray(c1, float), num, p, q, lag, samp,
                                        mtab, frametime, C.byref(ok), curve.ctypes.data)
    if want_curve:
        return ind, ok.value, curve.reshape(3, blocknum)
    return ind, ok.value


def calculate_cf(c0, c1, ind, p, q, gls=False):
    num = len(c0) - 1
    lag, samp, mtab = lag_tables(p, q, num)
    c = len(lag)
    corav = np.zeros(c)
    bv = np.zeros(c)
    bsd = np.zeros(c)
    cov = np.zeros((c - 1) * (c - 1)) if gls else None
    lib().imfcs_o_calculate_cf(np.ascontiguousarray(c0, float), np.ascontiguousarray(c1, float),
                               num, ind, p, q, lag, samp, mtab, int(gls), corav, bv, bsd,
                               None if cov is None else cov.ctypes.data)
    return corav, bv, bsd, (None if cov is None else cov.reshape(c - 1, c - 1))


def fcs_model(par, cst, tau, grad=False):
    v = C.c_double(0.0)
    g = np.zeros(NPARAM)
    lib().imfcs_o_fcs_model(np.ascontiguousarray(par, float), np.ascontiguousarray(cst, float),
                            float(tau), C.byref(v), g.ctypes.data if grad else None)
    return (v.value, g) if grad else v.value


def obsvol(ax, ay, s):
    return lib().imfcs_o_obsvol(ax, ay, s)


def fit_ols(acf, var, lagtime, fitstart, fitend, init, free_mask, cst, max_iter=2000):
    c = len(acf)
    out = np.zeros(NPARAM)
    x2 = C.c_double(0.0)
    it = C.c_int(0)
    k = int(np.sum(free_mask))
    cov = np.zeros(k * k)
    sig = np.zeros(k)
    tres = np.zeros(c - 1)
    st = lib().imfcs_o_fit_ols(np.ascontiguousarray(acf, float), np.ascontiguousarray(var, float),
                               np.ascontiguousarray(lagtime, float), c, fitstart, fitend,
                               np.ascontiguousarray(init, float),
                               np.ascontiguousarray(free_mask, np.int32),
                               np.ascontiguousarray(cst, float), max_iter, out, C.byref(x2),
                               cov.ctypes.data, sig.ctypes.data, tres.ctypes.data, C.byref(it))
    return dict(status=st, params=out, chi2=x2.value, cov=cov.reshape(k, k), sigma=sig,
                tres=tres, iters=it.value)


def fit_gls(acf, covmats, lagtime, init, free_mask, cst, max_iter=2000):
    c = len(acf)
    out = np.zeros(NPARAM)
    x2 = C.c_double(0.0)
    it = C.c_int(0)
    k = int(np.sum(free_mask))
    cov = np.zeros(k * k)
    sig = np.zeros(k)
    tres = np.zeros(c - 1)
    st = lib().imfcs_o_fit_gls(np.ascontiguousarray(acf, float),
                               np.ascontiguousarray(covmats, float).ravel(),
                               np.ascontiguousarray(lagtime, float), c,
                               np.ascontiguousarray(init, float),
                               np.ascontiguousarray(free_mask, np.int32),
                               np.ascontiguousarray(cst, float), max_iter, out, C.byref(x2),
                               cov.ctypes.data, sig.ctypes.data, tres.ctypes.data, C.byref(it))
    return dict(status=st, params=out, chi2=x2.value, cov=cov.reshape(k, k), sigma=sig,
                tres=tres, iters=it.value)


def bayes(acf, var, covmats, lagtime, fitstart, fitend, gls, init, cst, max_iter=2000):
    c = len(acf)
    prob = np.zeros(2)
    f1 = np.zeros(NPARAM)
    f2 = np.zeros(NPARAM)
    cm = None if covmats is None else np.ascontiguousarray(covmats, float).ravel()
    lib().imfcs_o_bayes(np.ascontiguousarray(acf, float), np.ascontiguousarray(var, float),
                        None if cm is None else cm.ctypes.data,
                        np.ascontiguousarray(lagtime, float), c, fitstart, fitend, int(gls),
                        np.ascontiguousarray(init, float), np.ascontiguousarray(cst, float),
                        max_iter, prob, f1, f2)
    return prob, f1, f2


def line_fit(x, y, sd):
    res = np.zeros(2)
    st = lib().imfcs_o_line_fit(np.ascontiguousarray(x, float), np.ascontiguousarray(y, float),
                                np.ascontiguousarray(sd, float), len(x), res)
    return res, st


def run(stack, *, out_w, out_h, map_x0=0, map_y0=0, binx=1, biny=1, pixbinx=None, pixbiny=None,
        cfx=0, cfy=0, background=0, p=16, q=8, frametime=1e-3, bleach=BLEACH_NONE, poly_order=0,
        gls=False, bayes=False, do_fit=True, fitstart=1, fitend=None, max_iter=2000,
        init=None, free_mask=None, cst=None, first=0, num=None, threads=0, bgr=None):
    """Whole CPU path over an output grid; returns a dict of numpy arrays."""
    stack = np.ascontiguousarray(stack, np.uint16)
    t, h, w = stack.shape
    num = t - first if num is None else num
    c = chanum(p, q)
    cfg = Config()
    cfg.width, cfg.height, cfg.frames = w, h, t
    cfg.first, cfg.num = first, num
    cfg.out_w, cfg.out_h, cfg.map_x0, cfg.map_y0 = out_w, out_h, map_x0, map_y0
    cfg.binx, cfg.biny = binx, biny
    cfg.pixbinx = binx if pixbinx is None else pixbinx
    cfg.pixbiny = biny if pixbiny is None else pixbiny
    cfg.cfx, cfg.cfy, cfg.background = cfx, cfy, background
    cfg.p, cfg.q, cfg.frametime = p, q, frametime
    cfg.bleach, cfg.poly_order = bleach, poly_order
    cfg.gls, cfg.bayes, cfg.do_fit = int(gls), int(bayes), int(do_fit)
    cfg.fitstart = fitstart
    cfg.fitend = c - 1 if fitend is None else fitend
    cfg.max_iter = max_iter
    init = np.zeros(NPARAM) if init is None else np.asarray(init, float)
    free_mask = np.zeros(NPARAM, np.int32) if free_mask is None else np.asarray(free_mask)
    cst = np.zeros(NCONST) if cst is None else np.asarray(cst, float)
    for i in range(NPARAM):
        cfg.init[i] = float(init[i])
        cfg.free_mask[i] = int(free_mask[i])
    for i in range(NCONST):
        cfg.cst[i] = float(cst[i])
    cfg.threads = threads
    n = out_w * out_h
    acf = np.zeros((n, c))
    var = np.zeros((n, c))
    sd = np.zeros((n, c))
    bind = np.zeros(n, np.int32)
    bok = np.zeros(n, np.int32)
    fitres = np.full((n, NPARAM), np.nan)
    chi2 = np.full(n, np.nan)
    fitted = np.zeros(n, np.int32)
    prob = np.zeros((n, 2))
    covmats = np.zeros((n, c - 1, c - 1)) if gls else None
    bgr_p = None if bgr is None else np.ascontiguousarray(bgr, np.int32).ctypes.data
    lib().imfcs_o_run(C.byref(cfg), stack, bgr_p, acf, var, sd, bind, bok, fitres, chi2, fitted,
                      prob.ctypes.data if bayes else None, None if covmats is None else covmats.ctypes.data)
    out = dict(acf=acf, var=var, sd=sd, blocked_ind=bind, blocked_ok=bok, fitres=fitres,
               chi2=chi2, fitted=fitted, bayes_prob=prob)
    if covmats is not None:
        out["covmats"] = covmats
    return out


def background_stats(stack):
    """loadBGRFile (Imaging_FCS_1_52.java:7036-7103) in FP64, in the Java's
    order: row and column means accumulated frame by frame as
    line_sum / (len * frames), the lag-1 covariance from the means of frames
    1..f-1 and 2..f, mean and variance over all frames.  Images are
    [height][width] (the Java's arrays are [x][y]).  Pixel values, squares and
    products are integers below 2^53, so every sum is exact."""
    st = np.asarray(stack).astype(np.float64)
    f, h, w = st.shape
    row = np.zeros(h)
    col = np.zeros(w)
    for z in range(f):
        row += st[z].sum(axis=1) / (w * f)
        col += st[z].sum(axis=0) / (h * f)
    m1 = st[:-1].sum(axis=0) / (f - 1)
    m2 = st[1:].sum(axis=0) / (f - 1)
    covar = (st[:-1] * st[1:]).sum(axis=0) / (f - 1) - m1 * m2
    mean = st.sum(axis=0) / f
    var = (st * st).sum(axis=0) / f - mean * mean
    return {"mean": mean, "var": var, "covar": covar, "row_mean": row, "col_mean": col}
