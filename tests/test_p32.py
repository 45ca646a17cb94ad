"""Correlator P = 32 (the plugin's cbCorrelatorP choice, java:1022-1024; lag
tables java:7391-7424: level 0 lags 0..32, then 16 lags per level) through
the plan and through the reference-facing calcACF, against the oracle:
blocking exactly, ACF within ACF_TOL of |G(1)|, blocked variance within
VAR_TOL, fitted N and D within FIT_TOL."""
import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib, engine
from tests.helpers import ACF_TOL, FIT_TOL, VAR_TOL, acf_deviation, run_both
from tests.synth import brownian_stack

W, H, T = 8, 7, 6000


def test_p32_channel_count_and_gls_limit():
    cfg = engine.FCSConfig(width=W, height=H, frames=T, p=32, q=8)
    assert cfg.chanum == 32 + 7 * 16 + 1
    # the GLS covariance of 144 lags does not fit one CTA: refused before
    # any device work
    with pytest.raises(_lib.ImfcsError, match="GLS"):
        engine.Plan(engine.FCSConfig(width=W, height=H, frames=T, p=32, q=8, gls=True))
    with pytest.raises(_lib.ImfcsError, match="P must be 16 or 32"):
        engine.Plan(engine.FCSConfig(width=W, height=H, frames=T, p=24, q=8))


@pytest.fixture(scope="module")
def bright():
    return brownian_stack(W, H, T, seed=41, density=2.0, cps=3e4, tau_bleach=8.0)


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [
    {"q": 8},
    {"q": 4},
    {"q": 8, "cfx": 1, "cfy": 1},
    {"q": 6, "binx": 2, "biny": 2},
    {"q": 8, "bleach": _lib.BLEACH_POLYNOMIAL, "poly_order": 4},
    {"q": 8, "bleach": _lib.BLEACH_SINGLE_EXP},
], ids=["q8", "q4", "ccf11", "bin2-q6", "poly4", "exp"])
def test_p32_matches_oracle(bright, kw):
    kw = dict(kw)
    cfg = engine.FCSConfig(width=W, height=H, frames=T, background=100, p=32, **kw)
    gpu, ref = run_both(bright, cfg)
    np.testing.assert_array_equal(gpu["blocked_ind"], ref["blocked_ind"])
    np.testing.assert_array_equal(gpu["blocked_ok"], ref["blocked_ok"])
    np.testing.assert_array_equal(np.isfinite(gpu["acf"]), np.isfinite(ref["acf"]))
    assert gpu["acf"].shape[1] == cfg.chanum
    assert acf_deviation(gpu, ref) <= ACF_TOL
    v_g, v_r = gpu["var"][:, 1:], ref["var"][:, 1:]
    fin = np.isfinite(v_r)
    rel = np.abs(v_g[fin] - v_r[fin]) / np.abs(v_r[fin])
    assert rel.max() <= VAR_TOL and np.median(rel) <= 1e-5
    if cfg.do_fit and not (cfg.cfx or cfg.cfy) and cfg.bleach != _lib.BLEACH_SINGLE_EXP:
        np.testing.assert_array_equal(gpu["fitted"], ref["fitted"])
        both = (gpu["fitted"] == 1) & (ref["fitted"] == 1)
        # (an order-4 bleach curve through zero leaves some pixels without
        # a finite correlation, in both)
        assert both.sum() >= 0.6 * cfg.npix
        for i in (0, 1):
            err = np.abs(gpu["fitres"][both, i] / ref["fitres"][both, i] - 1)
            assert err.max() <= FIT_TOL, (i, err.max())


@pytest.mark.gpu
def test_p32_reference_calc_acf(bright):
    """calcACF with correlatorp = 32 (agpufitjni.cu:5364, GpufitImFCS.java:533)
    on the float stack (background subtracted, no bleach correction): lag
    and sampling tables and the correlation against the oracle."""
    import ctypes as C
    import oracle
    L = _lib.load()
    q = 8
    ch = engine.FCSConfig(width=W, height=H, frames=T, p=32, q=q).chanum
    pixels = np.ascontiguousarray(bright.astype(np.float32) - 100.0)
    p = _lib.ACFParameters(width=W, height=H, win_star=W, hin_star=H, w_temp=W, h_temp=H, pixbinX=1, pixbinY=1,
                           binningX=1, binningY=1, firstframe=1, lastframe=T, framediff=T, cfXDistance=0,
                           cfYDistance=0, correlatorp=32, correlatorq=q, frametime=1e-3, background=100,
                           chanum=ch, isNBcalculation=0, bleachcorr_gpu=0, bleachcorr_order=0, nopit=1000,
                           ave=T // 1000)
    acf = np.zeros((ch, H, W))
    var = np.zeros_like(acf)
    blk = np.zeros((2, H, W))
    samp = np.zeros(ch)
    lag = np.zeros(ch, np.int32)
    rc = L.imfcs_calc_acf(pixels.ctypes.data, acf.ctypes.data, var.ctypes.data, None, None, blk.ctypes.data,
                          None, samp.ctypes.data, lag.ctypes.data, C.byref(p))
    assert rc == 0, _lib.last_error()
    lg, sp, _ = oracle.lag_tables(32, q, T)
    np.testing.assert_array_equal(lag, lg)
    np.testing.assert_array_equal(samp, sp)
    ref = oracle.run(bright, out_w=W, out_h=H, background=100, p=32, q=q, do_fit=False)
    g = acf.reshape(ch, -1).T
    np.testing.assert_array_equal(blk[0].ravel(), ref["blocked_ind"])
    np.testing.assert_array_equal(np.isfinite(g), np.isfinite(ref["acf"]))
    assert acf_deviation({"acf": g}, ref) <= ACF_TOL
