"""Host FCS_3p model (imaging_fcs_1_52_gb300.model, the workbook's fit
functions) against the oracle's restatement of the plugin's FCS_3p
(java:13131-13408), and the fit-function / residual rules of the plugin's
fits (java:10383-10397 OLS, 10701-10710 GLS)."""
import numpy as np
import pytest

import oracle
from imaging_fcs_1_52_gb300 import engine, model


def _random_params(rng, n):
    return np.column_stack([
        rng.uniform(0.5, 5, n), rng.uniform(0.1, 10, n) * 1e-12, rng.uniform(-50, 50, n) * 1e-6,
        rng.uniform(-50, 50, n) * 1e-6, rng.uniform(-0.01, 0.01, n), rng.uniform(0, 0.4, n),
        rng.uniform(1, 50, n) * 1e-12, rng.uniform(0, 0.3, n), rng.uniform(0.01, 0.5, n) * 1e-12,
        rng.uniform(0, 0.3, n), rng.uniform(1, 100, n) * 1e-6])


@pytest.mark.parametrize("binning,cfx,cfy,sz_um,q2", [
    (1, 0, 0, 1e6 * 0.515 / 1.49, 1.0),    # TIRF ACF
    (2, 1, 0, 1.2, 1.0),                   # SPIM (finite sz), CCF in x
    (3, 2, 1, 0.8, 0.6),                   # SPIM, diagonal CCF, dimmer component 2
])
def test_model_matches_oracle(binning, cfx, cfy, sz_um, q2):
    rng = np.random.default_rng(binning)
    lag, _ = engine.lag_tables(16, 8)
    tau = lag * 1e-3
    cst = engine.model_constants(binx=binning, biny=binning, cfx=cfx, cfy=cfy, sz_um=sz_um, q2=q2, q3=0.8)
    par = _random_params(rng, 6)
    got = model.fcs_model(par, cst, tau)
    for k in range(len(par)):
        want = np.array([oracle.fcs_model(par[k], cst, t) for t in tau])
        np.testing.assert_allclose(got[k], want, rtol=1e-12, atol=1e-15 * np.abs(want).max())


def test_model_triplet_time_zero():
    """Ttrip = 0: the triplet term vanishes at tau > 0 and the plugin's
    arithmetic gives NaN at tau = 0."""
    cst = engine.model_constants()
    par = np.array([2.0, 1e-12, 0, 0, 0, 0, 0, 0, 0, 0.2, 0.0])
    g = model.fcs_model(par, cst, np.array([0.0, 1e-3, 1e-2]))
    assert np.isnan(g[0]) and np.all(np.isfinite(g[1:]))
    ref = par.copy()
    ref[9] = 0.0
    np.testing.assert_allclose(g[1:], model.fcs_model(ref, cst, np.array([1e-3, 1e-2])), rtol=1e-15)


def test_fit_curves_ols_and_gls_rules():
    rng = np.random.default_rng(4)
    lag, _ = engine.lag_tables(16, 8)
    ch = len(lag)
    tau = lag * 1e-3
    cst = engine.model_constants()
    n = 5
    par = np.zeros((n, 11))
    par[:, 0] = rng.uniform(1, 3, n)
    par[:, 1] = rng.uniform(0.5, 3, n) * 1e-12
    par[:, 10] = 1e-6                           # Ttrip > 0: lag 0 finite (Ftrip = 0)
    truth = model.fcs_model(par, cst, tau)
    acf = truth + rng.normal(0, 1e-3, truth.shape)
    var = np.full((n, ch), 1e-6)
    fitted = np.array([1, 1, 0, 1, 1])
    fitres = par.copy()
    fitres[4, 1] = np.nan                       # a failed fit
    fit, res = model.fit_curves(acf, fitres, fitted, cst, tau, var=var, fitstart=3, fitend=60)
    for p in range(n):
        if p in (2, 4):
            assert not fit[p].any() and not res[p].any()
            continue
        assert not fit[p, :3].any() and not fit[p, 61:].any()
        np.testing.assert_allclose(fit[p, 3:61], truth[p, 3:61], rtol=1e-14)
        np.testing.assert_allclose(res[p, 3:61], (acf[p, 3:61] - truth[p, 3:61]) / 1e-3, rtol=1e-12)
    # GLS: every lag, residuals whitened by the covariance's Cholesky factor
    a = rng.normal(size=(n, ch - 1, ch - 1)) * 1e-4
    cov = a @ a.transpose(0, 2, 1) + np.eye(ch - 1) * 1e-6
    fit, res = model.fit_curves(acf, fitres, fitted, cst, tau, covmats=cov, gls=True)
    for p in (0, 1, 3):
        np.testing.assert_allclose(fit[p], truth[p], rtol=1e-14)
        assert res[p, 0] == pytest.approx(acf[p, 0] - truth[p, 0])
        low = np.linalg.cholesky(cov[p])
        np.testing.assert_allclose(low @ res[p, 1:], acf[p, 1:] - truth[p, 1:], rtol=1e-8, atol=1e-12)
