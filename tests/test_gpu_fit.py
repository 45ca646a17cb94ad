"""GPU parity of the fits through the C ABI: OLS (standardFit), GLS, Bayes,
the reference fit API (Gpufit ACF_1D / LINEAR_1D), the reference calcACF
path, and the diffusion law -- against the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle
from imaging_fcs_1_52_gb300 import _lib, engine
from tests.helpers import ACF_TOL, FIT_TOL, acf_deviation, oracle_kwargs, run_both
from tests.synth import brownian_stack

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bright():
    return brownian_stack(8, 8, 6000, seed=21, density=2.0, cps=3e4)


def fit_errors(gpu, ref, idx=(0, 1)):
    both = (gpu["fitted"] == 1) & (ref["fitted"] == 1)
    errs = {}
    for i in idx:
        errs[i] = np.abs(gpu["fitres"][both, i] - ref["fitres"][both, i]) / np.abs(ref["fitres"][both, i])
    return both, errs


def test_ols_fit_parity(bright):
    cfg = engine.FCSConfig(width=8, height=8, frames=6000, background=100)
    gpu, ref = run_both(bright, cfg)
    np.testing.assert_array_equal(gpu["fitted"], ref["fitted"])
    both, errs = fit_errors(gpu, ref)
    assert both.sum() >= 48
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL
    chi = np.abs(gpu["chi2"][both] - ref["chi2"][both]) / ref["chi2"][both]
    assert chi.max() <= 1e-3


def test_ols_fit_parity_poly_bleach_and_fit_range(bright):
    cfg = engine.FCSConfig(width=8, height=8, frames=6000, background=100, bleach=_lib.BLEACH_POLYNOMIAL,
                           poly_order=4, fitstart=2, fitend=60)
    gpu, ref = run_both(bright, cfg)
    assert acf_deviation(gpu, ref) <= ACF_TOL
    both, errs = fit_errors(gpu, ref)
    assert both.sum() >= 48
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL


def test_gls_fit_parity(bright):
    cfg = engine.FCSConfig(width=8, height=8, frames=6000, background=100, gls=True)
    gpu, ref = run_both(bright, cfg)
    # GLS hands over mcov (java:9638-9642); lag 0 is 0
    assert np.all(gpu["acf"][:, 0] == 0)
    assert acf_deviation(gpu, ref) <= ACF_TOL
    np.testing.assert_array_equal(gpu["fitted"], ref["fitted"])
    both, errs = fit_errors(gpu, ref)
    assert both.sum() >= 32
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL
    # the regularised covariance the fit whitens with (java:9524-9610), per
    # pixel relative to its largest element
    cg, cr = gpu["covmats"], ref["covmats"]
    fin = np.all(np.isfinite(cr.reshape(len(cr), -1)), axis=1)
    assert fin.sum() >= 32
    scale = np.abs(cr[fin]).reshape(fin.sum(), -1).max(axis=1)[:, None, None]
    assert np.max(np.abs(cg[fin] - cr[fin]) / scale) <= 1e-4


@pytest.mark.parametrize("kw", [{}, {"cfx": 1, "cfy": 0}], ids=["acf", "ccf10"])
def test_gls_long_stack_parity(kw):
    """20,000 frames: about 140 blocked products per lag, so the covariance
    pass runs over several staged chunks of samples."""
    st = brownian_stack(6, 5, 20000, seed=31, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(width=6, height=5, frames=20000, background=100, gls=True, **kw)
    gpu, ref = run_both(st, cfg)
    assert acf_deviation(gpu, ref) <= ACF_TOL
    cg, cr = gpu["covmats"], ref["covmats"]
    fin = np.all(np.isfinite(cr.reshape(len(cr), -1)), axis=1)
    assert fin.sum() >= 0.8 * len(cr)
    scale = np.abs(cr[fin]).reshape(fin.sum(), -1).max(axis=1)[:, None, None]
    assert np.max(np.abs(cg[fin] - cr[fin]) / scale) <= 1e-4
    np.testing.assert_array_equal(gpu["fitted"], ref["fitted"])
    both, errs = fit_errors(gpu, ref)
    assert both.sum() >= 0.8 * len(cr)
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL


def test_gls_covariance_many_ctas_matches_oracle():
    """A 96 x 4 strip of a two-component 20,000-frame stack: 384 pixels (a
    CTA each) with blocking indices 7..10, so the blocked products per lag
    (pnum) vary between neighbouring CTAs -- the covariance, its shrinkage
    and the whitened fit against the oracle on every pixel."""
    import torch
    full = engine.simulate(128, 16, 20000, d1=0.5, d2=5.0, fraction2=0.3, seed=3)
    st = engine.to_numpy_u16(full[:, :4, :96].contiguous())
    torch.cuda.synchronize()
    cfg = engine.batch_configs(96, 4, 20000, binnings=(1,), offsets=((0, 0),), background=100, gls=True)[0]
    gpu, ref = run_both(st, cfg)
    assert len(set(gpu["blocked_ind"].tolist())) >= 2
    cg, cr = gpu["covmats"], ref["covmats"]
    fin = np.all(np.isfinite(cr.reshape(len(cr), -1)), axis=1)
    assert fin.sum() >= 0.9 * len(cr)
    scale = np.abs(cr[fin]).reshape(fin.sum(), -1).max(axis=1)[:, None, None]
    assert np.max(np.abs(cg[fin] - cr[fin]) / scale) <= 1e-4
    np.testing.assert_array_equal(gpu["fitted"], ref["fitted"])
    both, errs = fit_errors(gpu, ref)
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL


@pytest.mark.parametrize("off,gls", [((1, 0), False), ((1, 1), False), ((0, 2), False), ((1, 0), True),
                                     ((1, 1), True)],
                         ids=["ccf10-ols", "ccf11-ols", "ccf02-ols", "ccf10-gls", "ccf11-gls"])
def test_ccf_fit_parity(off, gls):
    """Spatial cross-correlation fits with the window offsets in the model
    (rx, ry: the three-term lateral factor of FCS_3p, java:13131-13408),
    OLS and GLS, against the oracle.  Every pixel the oracle fits is fitted
    with N and D within FIT_TOL.  The weak correlations two pixels apart
    leave a few fits so flat that the oracle's LM stops at its 2000
    iterations (not fitted) where the GPU's Newton finish converges: at
    most 10 % of the pixels are fitted by the GPU alone.  (GLS at two
    pixels is left out: there D's standard error exceeds D on some pixels,
    and both optimisers stop within their step tolerances of a valley that
    flat, up to 5e-4 apart.)"""
    st = brownian_stack(8, 8, 8000, seed=33, density=3.0, cps=3e4)
    cfx, cfy = off
    cfg = engine.FCSConfig(width=8, height=8, frames=8000, background=100, cfx=cfx, cfy=cfy, gls=gls,
                           cst=engine.model_constants(cfx=cfx, cfy=cfy))
    gpu, ref = run_both(st, cfg)
    assert acf_deviation(gpu, ref) <= ACF_TOL
    assert np.all(gpu["fitted"][ref["fitted"] == 1] == 1)
    assert ((gpu["fitted"] == 1) & (ref["fitted"] == 0)).sum() <= 0.1 * cfg.npix
    both, errs = fit_errors(gpu, ref)
    assert both.sum() >= 0.5 * cfg.npix
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL
    rel = np.abs(gpu["chi2"][both] / ref["chi2"][both] - 1)
    assert rel.max() <= 1e-3


@pytest.fixture(scope="module")
def two_species():
    # 70 % of the particles at D = 0.5 um^2/s, 30 % at 5 um^2/s
    def d_map(x, y):
        return np.where(np.random.default_rng(4).random(len(x)) < 0.3, 5.0, 0.5)
    return brownian_stack(8, 8, 6000, seed=22, density=2.0, cps=3e4, d_map=d_map)


def test_bayes_probabilities(two_species):
    cfg = engine.FCSConfig(width=8, height=8, frames=6000, background=100, bayes=True)
    gpu, ref = run_both(two_species, cfg)
    p_g, p_r = gpu["bayes_prob"].astype(float), ref["bayes_prob"]
    # a two-component fit on a pixel that does not resolve the second
    # component has a singular covariance; that verdict (NaN) must agree on
    # most pixels, and the probabilities wherever both are finite
    ok_r, ok_g = np.all(np.isfinite(p_r), axis=1), np.all(np.isfinite(p_g), axis=1)
    assert (ok_r == ok_g).mean() >= 0.9
    ok = ok_r & ok_g
    assert ok.sum() >= 32
    np.testing.assert_allclose(p_g[ok].sum(1), 1.0, atol=1e-5)
    # same model choice on every pixel where the reference is decisive, and
    # the probabilities themselves
    dec = ok & (np.abs(p_r[:, 0] - 0.5) > 0.01)
    np.testing.assert_array_equal(p_g[dec, 0] > 0.5, p_r[dec, 0] > 0.5)
    assert np.max(np.abs(p_g[ok] - p_r[ok])) <= 1e-3


def _acf_curves(nfits, seed=0):
    lag, samp, mtab = oracle.lag_tables(16, 8, 50000)
    lagtime = lag * 1e-3
    cst = engine.model_constants()
    rng = np.random.default_rng(seed)
    data, var, truth = [], [], []
    for i in range(nfits):
        N, D = rng.uniform(2, 20), rng.uniform(0.3, 5) * 1e-12
        par = np.array([N, D, 0, 0, 0.001, 0, 0, 0, 0, 0, 0.0])
        g = np.array([oracle.fcs_model(par, cst, t) for t in lagtime])
        sd = 0.01 * np.abs(g[1]) + 0.02 * np.abs(g)
        data.append(g + rng.normal(0, 1, g.size) * sd)
        var.append(sd ** 2)
        truth.append(par)
    return np.array(data), np.array(var), lagtime, cst


def test_reference_fit_api_acf1d():
    L = _lib.load()
    n, npts = 40, 72
    data, var, lagtime, cst = _acf_curves(n)
    y = np.ascontiguousarray(data[:, 1:], np.float32)
    w = np.ascontiguousarray(1.0 / var[:, 1:], np.float32)
    init = np.zeros((n, 20), np.float32)
    init[:, 0], init[:, 1] = 1.0, 1e-12
    init[:, 11:20] = cst
    ptf = np.zeros(20, np.int32)
    ptf[[0, 1, 4]] = 1
    ui = np.ascontiguousarray(lagtime[1:], np.float32)
    outp = np.zeros((n, 20), np.float32)
    st = np.zeros(n, np.int32)
    chi = np.zeros(n, np.float32)
    it = np.zeros(n, np.int32)
    rc = L.imfcs_fit(n, npts, y.ctypes.data, w.ctypes.data, 2, init.ctypes.data, C.c_float(1e-16), 2000, 0,
                     ptf.ctypes.data, 0, ui.nbytes, ui.ctypes.data, outp.ctypes.data, st.ctypes.data,
                     chi.ctypes.data, it.ctypes.data)
    assert rc == 0, _lib.last_error()
    assert np.all(st == 0)
    np.testing.assert_array_equal(outp[:, 11:], init[:, 11:])   # constants pass through
    fm = np.array([1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0], np.int32)
    for i in range(n):
        r = oracle.fit_ols(data[i], var[i], lagtime, 1, 72, np.array([1, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0.0]), fm, cst)
        np.testing.assert_allclose(outp[i, [0, 1]], r["params"][[0, 1]], rtol=FIT_TOL)
        # chi-square: raw weighted sum of squares, as Gpufit returns it
        assert abs(chi[i] - r["chi2"] * (71 - 3 - 1)) <= 1e-3 * chi[i]


def test_reference_fit_api_linear1d():
    L = _lib.load()
    n, npts, ncoef = 16, 1000, 5
    rng = np.random.default_rng(3)
    x = np.ascontiguousarray(1e-3 * (np.arange(npts) + 0.5) * 20, np.float32)
    coefs = np.stack([rng.uniform(100, 500, n), rng.uniform(-5, -1, n), rng.uniform(0, .1, n),
                      rng.uniform(-1e-3, 0, n), rng.uniform(0, 1e-5, n)], 1)
    y = np.stack([np.polynomial.polynomial.polyval(x.astype(float), c) for c in coefs]) + rng.normal(0, 1, (n, npts))
    y = np.ascontiguousarray(y, np.float32)
    init = np.zeros((n, 11), np.float32)
    init[:, 0] = y[:, -1]
    ptf = np.zeros(11, np.int32)
    ptf[:ncoef] = 1
    outp = np.zeros((n, 11), np.float32)
    st = np.zeros(n, np.int32)
    rc = L.imfcs_fit(n, npts, y.ctypes.data, None, 3, init.ctypes.data, C.c_float(1e-6), 200, ncoef,
                     ptf.ctypes.data, 0, x.nbytes, x.ctypes.data, outp.ctypes.data, st.ctypes.data, None, None)
    assert rc == 0, _lib.last_error()
    for i in range(n):
        ref = np.polynomial.polynomial.polyfit(x.astype(float), y[i].astype(float), ncoef - 1)
        f_g = np.polynomial.polynomial.polyval(x.astype(float), outp[i, :ncoef].astype(float))
        f_r = np.polynomial.polynomial.polyval(x.astype(float), ref)
        assert np.max(np.abs(f_g - f_r)) <= 1e-3 * np.abs(f_r).max()


def test_reference_calc_acf_float_path():
    """calcACF: float stack [t][h_temp][w_temp] already binned and background
    subtracted, polynomial coefficients supplied per temp pixel."""
    L = _lib.load()
    raw = brownian_stack(9, 8, 4000, seed=31, density=2.0, cps=3e4)
    bx = by = 2
    wt, ht = 9 - bx + 1, 8 - by + 1
    f = raw.astype(np.float64)
    box = sum(f[:, j:j + ht, i:i + wt] for i in range(bx) for j in range(by)) - 100 * bx * by
    pixels = np.ascontiguousarray(box, np.float32)
    out_w, out_h, order = 3, 3, 4
    # per temp-pixel polynomial coefficients from the oracle's own bleach fit
    coef = np.zeros((ht, wt, order + 1))
    for y in range(ht):
        for x in range(wt):
            tr, tt = oracle.intensity_trace(raw, x, y, binx=bx, biny=by, bckg=100)
            coef[y, x], _ = oracle.poly_fit(tr, tt, order)
    p = _lib.ACFParameters(width=out_w, height=out_h, win_star=9, hin_star=8, w_temp=wt, h_temp=ht,
                           pixbinX=bx, pixbinY=by, binningX=bx, binningY=by, firstframe=1, lastframe=4000,
                           framediff=4000, cfXDistance=0, cfYDistance=0, correlatorp=16, correlatorq=8,
                           frametime=1e-3, background=100, chanum=73, isNBcalculation=0, bleachcorr_gpu=1,
                           bleachcorr_order=order + 1, nopit=1000, ave=4)
    acf = np.zeros((73, out_h, out_w))
    var = np.zeros_like(acf)
    blk = np.zeros((2, out_h, out_w))
    samp = np.zeros(73)
    lag = np.zeros(73, np.int32)
    cc = np.ascontiguousarray(coef)
    rc = L.imfcs_calc_acf(pixels.ctypes.data, acf.ctypes.data, var.ctypes.data, None, None, blk.ctypes.data,
                          cc.ctypes.data, samp.ctypes.data, lag.ctypes.data, C.byref(p))
    assert rc == 0, _lib.last_error()
    lg, sp, _ = oracle.lag_tables(16, 8, 4000)
    np.testing.assert_array_equal(lag, lg)
    np.testing.assert_array_equal(samp, sp)
    ref = oracle.run(raw, out_w=out_w, out_h=out_h, binx=bx, biny=by, background=100,
                     bleach=oracle.BLEACH_POLY, poly_order=order, do_fit=False)
    g = acf.reshape(73, -1).T
    np.testing.assert_array_equal(blk[0].ravel(), ref["blocked_ind"])
    # a polynomial bleach curve through zero makes exactly the lags whose
    # windows hold such a frame non-finite, in both
    np.testing.assert_array_equal(np.isfinite(g), np.isfinite(ref["acf"]))
    full = np.all(np.isfinite(ref["acf"]), axis=1)
    assert full.sum() >= 5
    assert acf_deviation({"acf": g}, ref) <= ACF_TOL


def test_reference_binning_and_bleach_average():
    L = _lib.load()
    rng = np.random.default_rng(5)
    frames, win, hin, bx, by = 100, 7, 6, 3, 2
    x = rng.integers(0, 50, (frames, hin, win)).astype(np.float32)
    wt, ht = win - bx + 1, hin - by + 1
    out = np.zeros((frames, ht, wt), np.float32)
    p = _lib.ACFParameters(win_star=win, hin_star=hin, w_temp=wt, h_temp=ht, binningX=bx, binningY=by,
                           pixbinX=1, pixbinY=1, firstframe=1, lastframe=frames, nopit=20, ave=5)
    assert L.imfcs_calc_binning(x.ctypes.data, out.ctypes.data, C.byref(p)) == 0
    ref = sum(x[:, j:j + ht, i:i + wt] for i in range(bx) for j in range(by))
    np.testing.assert_array_equal(out, ref)
    avg = np.zeros((ht, wt, 20), np.float32)
    assert L.imfcs_calc_data_bleach_correction(out.ctypes.data, avg.ctypes.data, C.byref(p)) == 0
    expect = np.trunc(out.reshape(20, 5, ht, wt).sum(1) / 5).transpose(1, 2, 0)
    np.testing.assert_array_equal(avg, expect)


def test_diffusion_law():
    import torch
    L = _lib.load()
    raw = brownian_stack(12, 12, 4000, seed=41, density=2.0, cps=3e4)
    dev = torch.from_numpy(raw.view(np.int16)).cuda().view(torch.uint16)
    cfg = engine.FCSConfig(width=12, height=12, frames=4000, background=100)
    c = cfg.to_c()
    out = np.zeros(9)
    line = np.zeros(2)
    rc = L.imfcs_diffusion_law(C.byref(c), C.c_void_p(dev.data_ptr()), 3, 1, 3, C.c_double(0.24e-6),
                               C.c_double(0.4e-6), out.ctypes.data_as(C.POINTER(C.c_double)),
                               line.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == 0, _lib.last_error()
    for u in (1, 2, 3):
        cst = engine.model_constants(binx=u, biny=u)
        r = oracle.run(raw, out_w=12 // u, out_h=12 // u, binx=u, biny=u, background=100,
                       init=np.array(cfg.init), free_mask=np.array(cfg.free_mask, np.int32), cst=cst)
        d = r["fitres"][r["fitted"] == 1, 1]
        mean, var = d.mean() * 1e12, (d ** 2).mean() * 1e24 - (d.mean() * 1e12) ** 2
        assert abs(out[3 * (u - 1)] - cst[6] * 1e12) <= 1e-9 * out[3 * (u - 1)]
        assert abs(out[3 * (u - 1) + 1] - mean) <= 1e-4 * mean
        assert abs(out[3 * (u - 1) + 2] - var) <= 1e-3 * abs(var) + 1e-6
    x = out[0::3]
    yv = x / out[1::3]
    sd = x / out[1::3] ** 2 * np.sqrt(out[2::3])
    ref, _ = oracle.line_fit(x, yv, sd)
    np.testing.assert_allclose(line, ref, rtol=1e-6)


def test_simulator_is_seeded_and_bleaches():
    import torch
    a = engine.simulate(16, 16, 3000, seed=7, tau_bleach=1.0, cps=1e5, density=2.0)
    b = engine.simulate(16, 16, 3000, seed=7, tau_bleach=1.0, cps=1e5, density=2.0)
    assert torch.equal(a.view(torch.int16), b.view(torch.int16))
    m = a.view(torch.int16).float().mean(dim=(1, 2)).cpu().numpy() - 100
    early, late = m[:300].mean(), m[-300:].mean()
    assert late < early * np.exp(-2.4) * 1.5   # ~exp(-t/tau) emission over 3 s


# ---------------------------------------------------------------------------
# FCS_3p model terms beyond the one-component TIRF case, through the
# reference fit API (Gpufit ACF_1D) against the oracle's standardFit: SPIM
# (finite sz), flow (vx, vy), triplet, a second and a third component, and
# the cross-correlation distance terms (rx, ry).
# ---------------------------------------------------------------------------
def _model_case(par, cst, free, init, nfits=12, seed=0, rel_noise=0.002):
    lag, _, _ = oracle.lag_tables(16, 8, 50000)
    lagtime = lag * 1e-3
    rng = np.random.default_rng(seed)
    data, var = [], []
    for i in range(nfits):
        p = np.array(par, float)
        p[0] *= rng.uniform(0.8, 1.25)
        p[1] *= rng.uniform(0.8, 1.25)
        g = np.array([oracle.fcs_model(p, cst, t) for t in lagtime])
        sd = rel_noise * np.abs(g[1]) + 0.01 * np.abs(g - p[4])
        data.append(g + rng.normal(0, 1, g.size) * sd)
        var.append(sd ** 2)
    return np.array(data), np.array(var), lagtime


def _fit_api_vs_oracle(par, cst, free, init, **kw):
    L = _lib.load()
    data, var, lagtime = _model_case(par, cst, free, init, **kw)
    n, npts = len(data), len(lagtime) - 1
    y = np.ascontiguousarray(data[:, 1:], np.float32)
    w = np.ascontiguousarray(1.0 / var[:, 1:], np.float32)
    ini = np.zeros((n, 20), np.float32)
    ini[:, :11] = init
    ini[:, 11:20] = cst
    ptf = np.zeros(20, np.int32)
    ptf[:11] = free
    ui = np.ascontiguousarray(lagtime[1:], np.float32)
    outp = np.zeros((n, 20), np.float32)
    st = np.zeros(n, np.int32)
    chi = np.zeros(n, np.float32)
    rc = L.imfcs_fit(n, npts, y.ctypes.data, w.ctypes.data, 2, ini.ctypes.data, C.c_float(1e-16), 2000, 0,
                     ptf.ctypes.data, 0, ui.nbytes, ui.ctypes.data, outp.ctypes.data, st.ctypes.data,
                     chi.ctypes.data, None)
    assert rc == 0, _lib.last_error()
    idx = np.flatnonzero(free)
    checked = 0
    for i in range(n):
        r = oracle.fit_ols(data[i], var[i], lagtime, 1, npts, np.array(init, float),
                           np.array(free, np.int32), cst)
        if r["status"] != 0:
            continue
        assert st[i] == 0
        for j in idx:
            # FIT_TOL relative, or 1e-4 of the parameter's standard error where
            # the fitted value is near zero (flow components)
            tol = max(FIT_TOL * abs(r["params"][j]), 1e-4 * r["sigma"][list(idx).index(j)])
            assert abs(outp[i, j] - r["params"][j]) <= tol, (i, j, outp[i, j], r["params"][j])
        assert abs(chi[i] - r["chi2"] * (npts - 1 - len(idx) - 1)) <= 1e-3 * chi[i]   # (fitend - fitstart) - K - 1
        checked += 1
    assert checked >= n // 2
    return checked


def _cst(sz=1e6 * 0.515 / 1.49 * 1e-6, rx=0.0, ry=0.0, q2=1.0, q3=1.0, s=0.4e-6):
    ax = ay = 0.24e-6
    return np.array([ax, ay, s, sz, rx, ry, oracle.obsvol(ax, ay, s), q2, q3])


ONE = [1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0]


def test_model_spim_finite_sz():
    par = [5.0, 2e-12, 0, 0, 0.001, 0, 0, 0, 0, 0, 0]
    _fit_api_vs_oracle(par, _cst(sz=0.9e-6), ONE, [1, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])


def test_model_flow():
    # flow along x free (with vx and vy both free on square pixels the
    # normal matrix is numerically singular: vy is not identifiable), and a
    # held flow along y
    par = [5.0, 1e-12, 2e-5, 0, 0.001, 0, 0, 0, 0, 0, 0]
    free = [1, 1, 1, 0, 1, 0, 0, 0, 0, 0, 0]
    _fit_api_vs_oracle(par, _cst(), free, [4, 1.2e-12, 1.5e-5, 0, 0, 0, 0, 0, 0, 0, 0], rel_noise=0.001)
    par = [5.0, 1e-12, 0, 1.5e-5, 0.001, 0, 0, 0, 0, 0, 0]
    _fit_api_vs_oracle(par, _cst(), ONE, [1, 1e-12, 0, 1.5e-5, 0, 0, 0, 0, 0, 0, 0])


def test_model_triplet_held_and_free():
    # a triplet time of a few lag times (1 ms frames), held and free
    par = [5.0, 2e-12, 0, 0, 0.001, 0, 0, 0, 0, 0.3, 3e-3]
    held = [1.0, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0.3, 3e-3]
    _fit_api_vs_oracle(par, _cst(), ONE, held)
    free = [1, 1, 0, 0, 1, 0, 0, 0, 0, 1, 1]
    _fit_api_vs_oracle(par, _cst(), free, [4, 1.5e-12, 0, 0, 0, 0, 0, 0, 0, 0.2, 2e-3], rel_noise=0.0005)


def test_model_two_components():
    par = [5.0, 0.5e-12, 0, 0, 0.001, 0.3, 8e-12, 0, 0, 0, 0]
    free = [1, 1, 0, 0, 1, 1, 1, 0, 0, 0, 0]
    _fit_api_vs_oracle(par, _cst(), free, [4, 0.6e-12, 0, 0, 0, 0.25, 6e-12, 0, 0, 0, 0], rel_noise=0.0005)


def test_model_third_component_and_brightness():
    par = [5.0, 0.5e-12, 0, 0, 0.001, 0.3, 5e-12, 0.2, 30e-12, 0, 0]
    held = [1, 1e-12, 0, 0, 0, 0.3, 5e-12, 0.2, 30e-12, 0, 0]
    _fit_api_vs_oracle(par, _cst(q2=1.5, q3=0.8), ONE, held)


def test_model_cross_correlation_distance():
    # the spatial CCF model at a one-pixel distance in x and in x and y
    par = [5.0, 3e-12, 0, 0, 0.0, 0, 0, 0, 0, 0, 0]
    _fit_api_vs_oracle(par, _cst(rx=0.24e-6), ONE, [4, 2e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    _fit_api_vs_oracle(par, _cst(rx=0.24e-6, ry=0.24e-6), ONE, [4, 2e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])


def test_plan_spim_fit_on_a_stack(bright):
    """The whole path with SPIM constants (finite sz) on a correlated stack."""
    cst = engine.model_constants(sz_um=0.9)
    cfg = engine.FCSConfig(width=8, height=8, frames=6000, background=100, cst=cst)
    gpu, ref = run_both(bright, cfg)
    np.testing.assert_array_equal(gpu["fitted"], ref["fitted"])
    both, errs = fit_errors(gpu, ref)
    assert both.sum() >= 48
    assert errs[0].max() <= FIT_TOL and errs[1].max() <= FIT_TOL


def test_reference_calc_acf_nb_mode():
    """N&B mode of calcACF (isNBcalculation, agpufitjni.cu:5719-5720): lag 1
    only -- NBmean = mean of the first num-1 samples, NBcov = <I(t) I(t+1)>
    minus the product of the two window means; the correlation outputs stay
    as passed.  Equal to the full path's N&B outputs and to numpy."""
    L = _lib.load()
    raw = brownian_stack(7, 6, 3000, seed=17, density=2.0, cps=3e4)
    pixels = np.ascontiguousarray(raw.astype(np.float32) - 100)
    base = dict(width=7, height=6, win_star=7, hin_star=6, w_temp=7, h_temp=6, pixbinX=1, pixbinY=1,
                binningX=1, binningY=1, firstframe=1, lastframe=3000, framediff=3000, cfXDistance=0,
                cfYDistance=0, correlatorp=16, correlatorq=8, frametime=1e-3, background=100, chanum=73,
                bleachcorr_gpu=0, bleachcorr_order=0, nopit=1000, ave=3)
    out = {}
    for nb in (0, 1):
        p = _lib.ACFParameters(isNBcalculation=nb, **base)
        acf = np.full(73 * 42, -7.0)
        m, c = np.zeros(42), np.zeros(42)
        rc = L.imfcs_calc_acf(pixels.ctypes.data, acf.ctypes.data, None, m.ctypes.data, c.ctypes.data, None, None,
                              None, None, C.byref(p))
        assert rc == 0, _lib.last_error()
        out[nb] = (acf, m, c)
    assert (out[1][0] == -7.0).all()                       # untouched in N&B mode
    np.testing.assert_allclose(out[1][1], out[0][1], rtol=1e-6)
    np.testing.assert_allclose(out[1][2], out[0][2], rtol=1e-5, atol=1e-6 * np.abs(out[0][2]).max())
    x = pixels.reshape(3000, 42).astype(np.float64)
    mean = x[:-1].mean(0)
    cov = (x[:-1] * x[1:]).mean(0) - mean * x[1:].mean(0)
    np.testing.assert_allclose(out[1][1], mean, rtol=1e-6)
    np.testing.assert_allclose(out[1][2], cov, rtol=1e-4, atol=1e-5 * np.abs(cov).max())


def test_async_host_path_matches_sync():
    """imfcs_plan_execute_host_async over a sequence of different stacks
    (two device stack buffers in turn, copies overlapping executions) gives
    what the synchronous host path gives for each."""
    import torch
    stacks = [brownian_stack(8, 6, 4000, seed=s, density=2.0, cps=3e4) for s in (51, 52, 53)]
    cfg = engine.FCSConfig(width=8, height=6, frames=4000, background=100, do_fit=True)
    plan = engine.Plan(cfg)
    try:
        ref = [plan.execute_host(st) for st in stacks]
        pinned = [torch.from_numpy(st.view(np.int16)).pin_memory().numpy().view(np.uint16) for st in stacks]
        outs = []
        for st in pinned:
            o = {}
            for n in engine.output_names(cfg):
                dt, shp = engine._OUT_SPEC[n]
                o[n] = np.zeros((cfg.npix, *shp(cfg.chanum)), dtype=dt)
            outs.append(o)
        # one output set per stack: results of earlier calls must not be
        # overwritten by later ones
        for st, o in zip(pinned, outs):
            plan.execute_host_async(st, o)
        plan.synchronize()
    finally:
        plan.close()
    for r, o in zip(ref, outs):
        for k in ("acf", "var", "blocked_ind", "fitres", "chi2", "fitted"):
            np.testing.assert_array_equal(o[k], r[k], err_msg=k)


def test_psf_calibration():
    """determinePSF (java:8115-8160): correlate once per binning, fit for
    every PSF size; mean D and the tabulated spread per (PSF, binning) as the
    oracle's fits give them."""
    import torch
    L = _lib.load()
    raw = brownian_stack(20, 20, 3000, seed=43, density=2.0, cps=3e4)
    dev = torch.from_numpy(raw.view(np.int16)).cuda().view(torch.uint16)
    cfg = engine.FCSConfig(width=20, height=20, frames=3000, background=100)
    c = cfg.to_c()
    psfs = np.array([0.35e-6, 0.4e-6, 0.45e-6])
    nbin, bin_start = 3, 2
    out = np.zeros((3, 3, nbin))
    rc = L.imfcs_psf_calibration(C.byref(c), C.c_void_p(dev.data_ptr()), nbin, bin_start,
                                 psfs.ctypes.data_as(C.POINTER(C.c_double)), 3, C.c_double(0.24e-6),
                                 out.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == 0, _lib.last_error()
    for ip, psf in enumerate(psfs):
        for u in range(nbin):
            b = u + 1
            cst = engine.model_constants(binx=b, biny=b, psf_um=psf * 1e6)
            r = oracle.run(raw, out_w=20 // b, out_h=20 // b, binx=b, biny=b, background=100,
                           init=np.array(cfg.init), free_mask=np.array(cfg.free_mask, np.int32), cst=cst)
            d = r["fitres"][r["fitted"] == 1, 1]
            mean = d.mean() * 1e12
            var = (d ** 2).mean() * 1e24 - mean ** 2
            cnt = 20 // b * 20 // b                # Java int arithmetic, left to right
            assert out[ip, 0, u] == u + bin_start
            assert abs(out[ip, 1, u] - mean) <= 1e-4 * mean
            assert abs(out[ip, 2, u] - var / np.sqrt(cnt)) <= 1e-3 * abs(var / np.sqrt(cnt)) + 1e-6
    # the fitted D depends on the assumed PSF
    assert out[0, 1, 0] != out[2, 1, 0]
    c_small = engine.FCSConfig(width=19, height=20, frames=3000, background=100).to_c()
    assert L.imfcs_psf_calibration(C.byref(c_small), C.c_void_p(dev.data_ptr()), 1, 1,
                                   psfs.ctypes.data_as(C.POINTER(C.c_double)), 1, C.c_double(0.24e-6),
                                   out.ctypes.data_as(C.POINTER(C.c_double)), None) != 0
    assert "20x20" in _lib.last_error()
