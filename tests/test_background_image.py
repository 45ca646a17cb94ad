"""Per-pixel background image (the plugin's background-file mode, bgrloaded:
getIntensity java:9671-9673, calcIntensityTrace java:9842-9845) through the
plan against the oracle, including the reference's subtraction of the
direct window's background from a cross-correlation's second averaged
trace."""
import numpy as np
import pytest

import oracle
from imaging_fcs_1_52_gb300 import _lib, engine
from tests.helpers import ACF_TOL, FIT_TOL, acf_deviation, oracle_kwargs
from tests.synth import brownian_stack


def _bg(h, w, seed):
    """A background image around the camera offset of the synthetic stacks
    (100): its rounded values are 99, 100 or 101 per pixel."""
    rng = np.random.default_rng(seed)
    return rng.uniform(98.6, 101.4, (h, w))


def test_oracle_ccf_trace_reads_direct_window_background():
    st = brownian_stack(4, 3, 2000, seed=2, density=2.0, cps=3e4)
    bg = np.floor(_bg(3, 4, 1) + 0.5).astype(np.int32)
    own, _ = oracle.intensity_trace(st, 2, 1, bckg=0, bgr=bg)
    other, _ = oracle.intensity_trace(st, 2, 1, bckg=0, bgr=bg, bg_window=(1, 1))
    # the averaged traces differ by the background difference of the windows
    # (int division of each average aside)
    assert np.abs((other - own) - (bg[1, 2] - bg[1, 1])).max() <= 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [
    {"bleach": _lib.BLEACH_SINGLE_EXP, "do_fit": True},
    {"cfx": 1, "bleach": _lib.BLEACH_POLYNOMIAL, "poly_order": 2},
    {"binx": 2, "biny": 2},
], ids=["acf-exp-fit", "ccf10-poly", "bin2"])
def test_background_image_matches_oracle(kw):
    w, h, t = 10, 8, 6000
    st = brownian_stack(w, h, t, seed=13, density=2.0, cps=3e4, tau_bleach=20.0)
    bg = _bg(h, w, 7)
    bgr = np.floor(bg + 0.5).astype(np.int32)          # Math.round
    cfg = engine.FCSConfig(width=w, height=h, frames=t, background=100, **kw)
    plan = engine.Plan(cfg)
    try:
        plan.set_background_image(bg)
        gpu = plan.execute_host(st)
        plan.set_background_image(None)
        scalar = plan.execute_host(st)
    finally:
        plan.close()
    ref = oracle.run(st, **oracle_kwargs(cfg), bgr=bgr)
    np.testing.assert_array_equal(gpu["blocked_ind"], ref["blocked_ind"])
    np.testing.assert_array_equal(np.isfinite(gpu["acf"]), np.isfinite(ref["acf"]))
    assert acf_deviation(gpu, ref) <= ACF_TOL
    # the image changed the result (it is not the scalar background)
    fin = np.isfinite(gpu["acf"]) & np.isfinite(scalar["acf"])
    assert np.abs(gpu["acf"][fin] - scalar["acf"][fin]).max() > 100 * ACF_TOL * np.abs(gpu["acf"][fin]).max()
    if cfg.do_fit:
        both = (gpu["fitted"] == 1) & (ref["fitted"] == 1)
        assert both.sum() >= 0.8 * cfg.npix
        for i in (0, 1):
            rel = np.abs(gpu["fitres"][both, i] / ref["fitres"][both, i] - 1)
            assert rel.max() <= FIT_TOL, (i, rel.max())


@pytest.mark.gpu
def test_background_image_rejects_bad_input():
    cfg = engine.FCSConfig(width=6, height=5, frames=3000, background=100)
    plan = engine.Plan(cfg)
    try:
        with pytest.raises(ValueError):
            plan.set_background_image(np.zeros((4, 6)))
        bad = np.full((5, 6), 100.0)
        bad[2, 3] = np.nan
        with pytest.raises(_lib.ImfcsError):
            plan.set_background_image(bad)
    finally:
        plan.close()
