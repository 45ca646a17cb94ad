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


def acf_deviation(gpu, ref):
    """max over pixels and lags >= 1 of |dG| / |G(lag 1)| (finite pixels)."""
    a_g, a_r = gpu["acf"][:, 1:], ref["acf"][:, 1:]
    scale = np.abs(ref["acf"][:, 1:2])
    ok = np.all(np.isfinite(a_r), axis=1)
    return float(np.max(np.abs(a_g[ok] - a_r[ok]) / scale[ok])) if ok.any() else 0.0
