"""Shared helpers: run the same configuration through the GPU engine (C ABI)
and through the FP64 oracle."""
import numpy as np

import oracle
from imaging_fcs_1_52_gb300 import engine

# Tolerances, stated once (FP32 GPU path vs FP64 oracle):
ACF_TOL = 1e-5      # |dG| <= ACF_TOL * |G(lag 1)| for every lag >= 1
VAR_TOL = 5e-4      # relative, blocked variance (max); the median is checked at 1e-5
FIT_TOL = 1e-4      # relative, fitted N and D


def oracle_kwargs(cfg):
    return dict(out_w=cfg.out_w, out_h=cfg.out_h, map_x0=cfg.map_x0, map_y0=cfg.map_y0, binx=cfg.binx,
                biny=cfg.biny, pixbinx=cfg.pixbinx, pixbiny=cfg.pixbiny, cfx=cfg.cfx, cfy=cfg.cfy,
                background=cfg.background, p=cfg.p, q=cfg.q, frametime=cfg.frametime, bleach=cfg.bleach,
                poly_order=cfg.poly_order, gls=cfg.gls, bayes=cfg.bayes, do_fit=cfg.do_fit,
                fitstart=cfg.fitstart, fitend=cfg.fitend, max_iter=cfg.max_iter, init=np.array(cfg.init),
                free_mask=np.array(cfg.free_mask, np.int32), cst=cfg.cst, first=cfg.first, num=cfg.num)


def run_both(stack, cfg):
    gpu = engine.run_host(stack, cfg)
    ref = oracle.run(stack, **oracle_kwargs(cfg))
    return gpu, ref


def acf_scale(ref_acf):
    """Per-pixel scale of the ACF tolerance: |G(lag 1)|, or, where lag 1 is
    not finite (a non-finite frame in its windows), the largest finite |G|
    of lags >= 1."""
    a = np.abs(ref_acf[:, 1:])
    g1 = a[:, 0]
    alt = np.where(np.isfinite(a), a, 0.0).max(axis=1)
    return np.where(np.isfinite(g1), g1, alt)[:, None]


def acf_deviation(gpu, ref):
    """max over pixels and lags >= 1 of |dG| / scale (entries finite in the
    reference; see acf_scale)."""
    a_g, a_r = gpu["acf"][:, 1:], ref["acf"][:, 1:]
    fin = np.isfinite(a_r)
    if not fin.any():
        return 0.0
    dev = np.abs(a_g - a_r) / acf_scale(ref["acf"])
    return float(np.max(dev[fin]))
