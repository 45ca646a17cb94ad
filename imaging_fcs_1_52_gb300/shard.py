"""Pixel sharding across ranks (one process per GPU).

Output pixels are independent, so a job splits into contiguous bands of
output rows with no data exchange: each rank reads its band plus the halo
its windows need ((binning - 1) + |cfy| rows, duplicated at load).  The only
reduction is the diffusion law's (count, sum D, sum D^2) per binning.
"""
from __future__ import annotations

import dataclasses

import numpy as np


def shard_rows(out_h: int, world: int, rank: int) -> tuple[int, int]:
    """(first output row, number of rows) of `rank`'s band; bands differ by at most one row."""
    base, extra = divmod(out_h, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def shard_config(cfg, world: int, rank: int):
    """The rank's part of a job: same stack, map_y0 shifted to its band."""
    y0, rows = shard_rows(cfg.out_h, world, rank)
    return dataclasses.replace(cfg, map_y0=cfg.map_y0 + y0, out_h=rows)


def diffusion_partials(fitres: np.ndarray, fitted: np.ndarray) -> np.ndarray:
    """(count, sum D, sum D^2) of the fitted pixels (java:11175-11189), SI units."""
    d = fitres[fitted.astype(bool), 1].astype(np.float64)
    return np.array([d.size, d.sum(), (d * d).sum()])


def diffusion_point(partials: np.ndarray) -> tuple[float, float]:
    """Mean D [um^2/s] and variance of D from reduced partials (java:11189-11191).
    A binning without a fitted pixel gives (nan, nan), as the reference's
    0/0 does (java:11187-11189)."""
    n, s, s2 = partials
    if n == 0:
        return float("nan"), float("nan")
    mean = s * 1e12 / n
    return mean, s2 * 1e24 / n - mean * mean
