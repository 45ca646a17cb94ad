"""CPU tests of the FP64 oracle: documented known answers, analytic cases,
an independent numpy restatement of the correlator, and MINPACK (scipy)
for the least-squares minima."""
import math

import numpy as np
import pytest

import oracle
from tests.synth import brownian_stack

TIRF_SZ = 1e6 * 515 / 1.49 * 1e-9


def tirf_consts(px=0.24e-6, s=0.4e-6):
    return np.array([px, px, s, TIRF_SZ, 0, 0, oracle.obsvol(px, px, s), 1, 1])


# ---------------------------------------------------------------- lag tables
def test_lag_table_documented_example():
    # Reference manual, chapter 2 "Correlator P/Q": P=16, Q=6 gives lags 1..16,
    # then 18..32 step 2, 36..64 step 4, 72..128 step 8, 144..256 step 16, ...
    lag, samp, mtab = oracle.lag_tables(16, 6, 10000)
    assert len(lag) == oracle.chanum(16, 6) == 16 + 5 * 8 + 1
    assert list(lag[:17]) == list(range(17))
    assert list(lag[17:25]) == list(range(18, 33, 2))
    assert list(lag[25:33]) == list(range(36, 65, 4))
    assert list(lag[33:41]) == list(range(72, 129, 8))
    assert list(lag[41:49]) == list(range(144, 257, 16))
    assert list(samp[:17]) == [1] * 17
    assert list(samp[17:25]) == [2] * 8
    assert mtab[0] == 10000 and mtab[17] == (10000 - 18) // 2


@pytest.mark.parametrize("p,q,c", [(16, 8, 73), (16, 7, 65), (32, 8, 145), (16, 1, 17)])
def test_chanum(p, q, c):
    assert oracle.chanum(p, q) == c


# -------------------------------------------------- numpy restatement of the CF
def np_block_transform(c0, c1, p, q, lag, samp, mtab):
    num = len(c0) - 1
    blocknum = int(math.floor(math.log(mtab[1]) / math.log(2))) - 2
    x0 = np.asarray(c0[:num], float)
    x1 = np.asarray(c1[:num], float)
    d = x0[:-1]
    e = x1[1:]
    dm, Dm = d.mean(), e.mean()
    prod = d * e - Dm * d - dm * e + Dm * dm
    n0 = len(prod)
    sd = []
    pn = []
    for y in range(blocknum):
        n = n0 >> y
        blk = prod[: n << y].reshape(n, 1 << y).mean(axis=1)
        v = (np.mean(blk ** 2) - np.mean(blk) ** 2) / (n * (dm * Dm) ** 2)
        sd.append(math.sqrt(v) if v >= 0 else float("nan"))
        pn.append(n)
    sd = np.array(sd)
    err = sd / np.sqrt(2 * (np.array(pn) - 1))
    up, lo = sd + err, sd - err
    crt = [(up[x] > lo[x + 1]) and (up[x + 1] > lo[x]) for x in range(blocknum - 1)]
    cr12 = [int(crt[x] and crt[x + 1]) for x in range(blocknum - 2)]
    dpos = [sd[x + 1] - sd[x] > 0 for x in range(blocknum - 1)]
    cr3 = [int(dpos[x] and dpos[x + 1]) for x in range(blocknum - 2)]
    last0 = 0
    for x in range(blocknum - 2):
        if cr3[x] == 1 and cr12[x] == 0:
            last0 = x
    for x in range(last0 + 1):
        cr12[x] = 0
    cr12[blocknum - 3] = 0
    cr12[blocknum - 4] = 0
    ind = 0
    for x in range(blocknum - 5, 0, -1):
        if cr12[x] == 1:
            ind = x + 1
    ok = 1
    if ind == 0:
        ok = 0
        ind = blocknum - 3 if blocknum - 3 > 0 else blocknum - 1
    return max(ind, q - 1), ok


def np_calculate_cf(c0, c1, ind, p, q, lag, samp, mtab):
    chanum = len(lag)
    num = len(c0) - 1
    pnum = int(math.floor(mtab[-1] / 2 ** max(ind - math.log(samp[-1]) / math.log(2), 0)))
    a = np.asarray(c0[1:], float)
    b = np.asarray(c1[1:], float)
    cur, ctbin = 1, 0
    corav, bvar = np.zeros(chanum), np.zeros(chanum)
    for x in range(chanum):
        if cur != samp[x]:
            n = len(a) // 2
            a = a[: 2 * n].reshape(n, 2).sum(1)
            b = b[: 2 * n].reshape(n, 2).sum(1)
            cur = int(samp[x])
            ctbin += 1
        dl = lag[x] // cur
        pn = len(a) - dl
        d, e = a[:pn], b[dl:dl + pn]
        dm, Dm = d.mean(), e.mean()
        prod = (d - dm) * (e - Dm)
        corav[x] = prod.sum() / (pn * dm * Dm)
        L = 1 << (ind - ctbin)
        blk = prod[: pnum * L].reshape(pnum, L).mean(1)
        bvar[x] = (np.mean(blk ** 2) - np.mean(blk) ** 2) / ((pnum - 1) * (dm * Dm) ** 2)
    return corav, bvar


@pytest.mark.parametrize("frames,q", [(2200, 8), (6000, 8), (5000, 6)])
def test_correlator_matches_numpy_restatement(frames, q):
    st = brownian_stack(3, 3, frames, seed=frames + q, density=2.0)
    lag, samp, mtab = oracle.lag_tables(16, q, frames)
    for px, py in ((0, 0), (1, 2)):
        c = oracle.get_intensity(st, px, py, bckg=100)
        ind, ok = oracle.block_transform(c, c, 16, q)
        ind_np, ok_np = np_block_transform(c, c, 16, q, lag, samp, mtab)
        assert (ind, ok) == (ind_np, ok_np)
        corav, bv, bsd, _ = oracle.calculate_cf(c, c, ind, 16, q)
        corav_np, bv_np = np_calculate_cf(c, c, ind, 16, q, lag, samp, mtab)
        np.testing.assert_allclose(corav, corav_np, rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(bv, bv_np, rtol=1e-7, atol=1e-18)
        np.testing.assert_allclose(bsd, np.sqrt(bv), rtol=1e-12)


def test_ccf_matches_numpy_restatement():
    st = brownian_stack(4, 3, 3000, seed=9, density=2.0)
    lag, samp, mtab = oracle.lag_tables(16, 8, 3000)
    c0 = oracle.get_intensity(st, 0, 0, bckg=100)
    c1 = oracle.get_intensity(st, 1, 0, bckg=100)
    ind, ok = oracle.block_transform(c0, c1, 16, 8)
    assert (ind, ok) == np_block_transform(c0, c1, 16, 8, lag, samp, mtab)
    corav, bv, _, _ = oracle.calculate_cf(c0, c1, ind, 16, 8)
    corav_np, bv_np = np_calculate_cf(c0, c1, ind, 16, 8, lag, samp, mtab)
    np.testing.assert_allclose(corav, corav_np, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(bv, bv_np, rtol=1e-7, atol=1e-18)


def test_constant_trace_gives_zero_correlation():
    c = np.full(3001, 250.0)
    c[0] = 0.0
    corav, bv, _, _ = oracle.calculate_cf(c, c, 7, 16, 8)
    assert np.all(corav == 0.0)
    assert np.all(bv == 0.0)


def test_poisson_white_noise():
    rng = np.random.default_rng(4)
    mu = 50.0
    c = np.concatenate([[0.0], rng.poisson(mu, 40000).astype(float)])
    ind, ok = oracle.block_transform(c, c, 16, 8)
    corav, bv, bsd, _ = oracle.calculate_cf(c, c, ind, 16, 8)
    assert abs(corav[0] - 1 / mu) < 5 * bsd[0] + 1e-3
    assert np.all(np.abs(corav[1:]) < 6 * bsd[1:])


def test_binning_and_background():
    st = brownian_stack(6, 6, 100, seed=2)
    c = oracle.get_intensity(st, 1, 2, binx=3, biny=2, bckg=100)
    ref = st[:, 2:4, 1:4].astype(int).sum(axis=(1, 2)) - 100 * 6
    assert c[0] == 0.0
    np.testing.assert_array_equal(c[1:], ref)


def test_intensity_trace_int_division():
    st = brownian_stack(3, 3, 2500, seed=3)
    tr, tt = oracle.intensity_trace(st, 1, 1, bckg=101, frametime=1e-3)
    ave = 2500 // 1000
    raw = st[: 1000 * ave, 1, 1].astype(int) - 101
    sums = raw.reshape(1000, ave).sum(1)
    expect = np.trunc(sums / ave)   # Java int division truncates toward zero
    np.testing.assert_array_equal(tr, expect)
    np.testing.assert_allclose(tt, 1e-3 * (np.arange(1000) + 0.5) * ave)


# ------------------------------------------------------------------ bleach fits
def test_poly_fit_matches_numpy():
    t = 1e-3 * (np.arange(1000) + 0.5) * 20
    rng = np.random.default_rng(1)
    y = 500 - 3.0 * t + 0.05 * t ** 2 - 0.001 * t ** 3 + rng.normal(0, 2, t.size)
    for order in (1, 2, 4, 6):
        coef, st = oracle.poly_fit(y, t, order)
        assert st == 0
        ref = np.polynomial.polynomial.polyfit(t, y, order)
        fit_o = np.polynomial.polynomial.polyval(t, coef)
        fit_r = np.polynomial.polynomial.polyval(t, ref)
        np.testing.assert_allclose(fit_o, fit_r, rtol=1e-10, atol=1e-8)


def test_exp_fit_matches_scipy():
    from scipy.optimize import least_squares
    t = 1e-3 * (np.arange(1000) + 0.5) * 50
    rng = np.random.default_rng(2)
    y = 300 * np.exp(-t / 20.0) + 100 + rng.normal(0, 1.5, t.size)
    res, st = oracle.exp_fit(y, t)
    assert st == 0
    r = least_squares(lambda p: p[0] * np.exp(-t / p[1]) + p[2] - y, [y[1], t[500], 0], method="lm",
                      xtol=1e-15, ftol=1e-15, gtol=1e-15)
    np.testing.assert_allclose(res, r.x, rtol=1e-6)


def test_bleach_correction_formula():
    intdat = np.concatenate([[0.0], np.full(100, 80.0)])
    res = np.array([50.0, 2.0, 30.0])
    out = oracle.bleach_apply(intdat, 1e-3, oracle.BLEACH_SINGLE_EXP, res)
    x = np.arange(1, 101)
    f = (50 * np.exp(-1e-3 * (x + 0.5) / 2.0) + 30) / 80.0
    np.testing.assert_allclose(out[1:], 80 / np.sqrt(f) + 80 * (1 - np.sqrt(f)), rtol=1e-14)


# -------------------------------------------------------------------- the model
def test_model_gradient_matches_finite_differences():
    cst = np.array([0.24e-6, 0.24e-6, 0.4e-6, 1.2e-6, 0.1e-6, 0.05e-6, oracle.obsvol(0.24e-6, 0.24e-6, 0.4e-6), 1.3, 0.7])
    par = np.array([5.0, 2e-12, 1e-5, -2e-5, 0.01, 0.3, 8e-12, 0.2, 0.5e-12, 0.1, 5e-3])
    for tau in (1e-3, 3e-2, 0.5):
        v, g = oracle.fcs_model(par, cst, tau, grad=True)
        for i in range(11):
            h = abs(par[i]) * 1e-6 + 1e-20
            pp, pm = par.copy(), par.copy()
            pp[i] += h
            pm[i] -= h
            fd = (oracle.fcs_model(pp, cst, tau) - oracle.fcs_model(pm, cst, tau)) / (2 * h)
            assert abs(g[i] - fd) <= 1e-5 * abs(fd) + 1e-8 * abs(v) / abs(par[i]), (i, tau, g[i], fd)


def test_model_closed_form_tirf():
    # one component, no flow, TIRF: G = (1/N) Lx Ly / (4 ax^2 ay^2 / fitobsvol) + Ginf
    ax, s = 0.24e-6, 0.4e-6
    cst = tirf_consts(ax, s)
    N, D, G = 4.0, 1.5e-12, 0.002
    par = np.array([N, D, 0, 0, G, 0, 0, 0, 0, 0, 0.0])
    for tau in (1e-3, 0.01, 0.3):
        p0 = math.sqrt(4 * D * tau + s * s)
        L = p0 / math.sqrt(3.14159265359) * (2 * math.exp(-(ax / p0) ** 2) - 2) + 2 * ax * math.erf(ax / p0)
        expect = L * L / (4 * ax ** 4 / cst[6]) / N / math.sqrt(1 + 4 * D * tau / TIRF_SZ ** 2) + G
        assert abs(oracle.fcs_model(par, cst, tau) - expect) < 1e-12 * abs(expect)


def test_obsvol_limit():
    # tiny PSF: the observation area tends to the pixel area ax*ay
    ax = 1e-6
    assert abs(oracle.obsvol(ax, ax, 1e-9) - ax * ax) / (ax * ax) < 1e-2


# ------------------------------------------------------------------------- fits
def synth_acf(N=8.0, D=1.2e-12, G=0.003, noise=0.002, seed=0):
    lag, samp, mtab = oracle.lag_tables(16, 8, 50000)
    lagtime = lag * 1e-3
    cst = tirf_consts()
    par = np.array([N, D, 0, 0, G, 0, 0, 0, 0, 0, 0.0])
    g = np.array([oracle.fcs_model(par, cst, t) for t in lagtime])
    rng = np.random.default_rng(seed)
    sd = noise * np.abs(g) + 1e-4
    acf = g + rng.normal(0, 1, g.size) * sd
    return acf, sd ** 2, lagtime, cst


def test_ols_fit_matches_minpack():
    from scipy.optimize import least_squares
    acf, var, lagtime, cst = synth_acf()
    init = np.array([1.0, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    fm = np.array([1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0], np.int32)
    r = oracle.fit_ols(acf, var, lagtime, 1, 72, init, fm, cst)
    assert r["status"] == 0
    w = 1 / np.sqrt(var[1:])

    def resid(p):
        par = np.array([p[0], p[1] * 1e-12, 0, 0, p[2], 0, 0, 0, 0, 0, 0])
        return (np.array([oracle.fcs_model(par, cst, t) for t in lagtime[1:]]) - acf[1:]) * w

    s = least_squares(resid, [1.0, 1.0, 0.0], method="lm", xtol=1e-15, ftol=1e-15, gtol=1e-15)
    got = r["params"][[0, 1, 4]] * np.array([1, 1e12, 1])
    np.testing.assert_allclose(got, s.x, rtol=1e-7, atol=1e-10)
    chi2 = np.sum(resid(s.x) ** 2) / (71 - 3 - 1)
    assert abs(r["chi2"] - chi2) < 1e-9 * chi2


def test_gls_with_diagonal_covariance_equals_ols():
    acf, var, lagtime, cst = synth_acf(seed=3)
    init = np.array([1.0, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    fm = np.array([1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0], np.int32)
    o = oracle.fit_ols(acf, var, lagtime, 1, 72, init, fm, cst)
    g = oracle.fit_gls(acf, np.diag(var[1:]), lagtime, init, fm, cst)
    assert o["status"] == 0 and g["status"] == 0
    np.testing.assert_allclose(g["params"], o["params"], rtol=1e-7)


def test_bayes_probabilities():
    # data from two components: the two-component model must win
    lag, samp, mtab = oracle.lag_tables(16, 8, 50000)
    lagtime = lag * 1e-3
    cst = tirf_consts()
    par = np.array([6.0, 0.5e-12, 0, 0, 0.001, 0.4, 8e-12, 0, 0, 0, 0.0])
    g = np.array([oracle.fcs_model(par, cst, t) for t in lagtime])
    rng = np.random.default_rng(7)
    sd = 0.002 * np.abs(g) + 2e-5
    acf = g + rng.normal(0, 1, g.size) * sd
    init = np.array([1.0, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    prob, f1, f2 = oracle.bayes(acf, sd ** 2, None, lagtime, 1, 72, False, init, cst)
    assert np.all(np.isfinite(prob))
    assert abs(prob.sum() - 1) < 1e-12
    np.testing.assert_allclose(np.sort(f2[[1, 6]]), [0.5e-12, 8e-12], rtol=0.05)   # labels may swap
    # recompute java:10171-10207 from the two fits: with OLS the residual term
    # uses the unweighted residuals from index 1 on
    lp = []
    for k, fm, i5 in ((3, [1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0], None), (5, [1, 1, 0, 0, 1, 1, 1, 0, 0, 0, 0], 1)):
        ii = init.copy()
        if i5:
            ii[5], ii[6] = 0.5, 0.1 * init[1]
        r = oracle.fit_ols(acf, sd ** 2, lagtime, 1, 72, ii, np.array(fm, np.int32), cst)
        logresid = -0.5 * np.sum(r["tres"][1:] ** 2)
        lp.append(0.5 * k * math.log(2 * 3.14159265359) + 0.5 * math.log(np.linalg.det(r["cov"])) + logresid
                  - math.log(np.prod(r["sigma"]) * 400.0 ** k))
    p1 = 1 / (1 + math.exp(lp[1] - lp[0]))
    assert abs(prob[0] - p1) < 1e-9


def test_line_fit_weighted():
    x = np.array([0.1, 0.2, 0.35, 0.5, 0.8])
    y = 0.05 + 0.9 * x + np.array([0.001, -0.002, 0.0015, 0.0, -0.001])
    sd = np.array([0.01, 0.02, 0.01, 0.03, 0.02])
    res, st = oracle.line_fit(x, y, sd)
    ref = np.polyfit(x, y, 1, w=1 / sd)
    np.testing.assert_allclose(res, ref[::-1], rtol=1e-9)


def test_run_grid_equals_single_pixel_calls():
    st = brownian_stack(4, 4, 3000, seed=6)
    cst = tirf_consts()
    init = np.array([1.0, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    fm = np.array([1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0], np.int32)
    r = oracle.run(st, out_w=2, out_h=2, binx=2, biny=2, background=100, init=init, free_mask=fm, cst=cst,
                   bleach=oracle.BLEACH_POLY, poly_order=3)
    c = oracle.get_intensity(st, 2, 2, binx=2, biny=2, bckg=100)
    tr, tt = oracle.intensity_trace(st, 2, 2, binx=2, biny=2, bckg=100)
    coef, _ = oracle.poly_fit(tr, tt, 3)
    c = oracle.bleach_apply(c, 1e-3, oracle.BLEACH_POLY, coef, 3)
    ind, ok = oracle.block_transform(c, c, 16, 8)
    corav, bv, _, _ = oracle.calculate_cf(c, c, ind, 16, 8)
    np.testing.assert_array_equal(r["acf"][3], corav)
    np.testing.assert_array_equal(r["var"][3], bv)
    assert r["blocked_ind"][3] == ind
