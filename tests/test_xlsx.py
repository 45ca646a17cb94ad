"""Results writer in the plugin's .xlsx layout (java:4419-5020): sheet order
and names, the per-pixel column scheme (w + h * width), lag table and fit
parameter rows, read back with the standard library."""
import re
import zipfile
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import engine, xlsx

NS = {"m": "http://schemas.openxmlformats.org/spreadsheetml/2006/main"}


def read_xlsx(path):
    """{sheet name: {(row, col): value}} with 0-based indices."""
    out = {}
    with zipfile.ZipFile(path) as z:
        wb = ET.fromstring(z.read("xl/workbook.xml"))
        names = [s.get("name") for s in wb.find("m:sheets", NS)]
        for i, name in enumerate(names):
            sh = ET.fromstring(z.read(f"xl/worksheets/sheet{i + 1}.xml"))
            cells = {}
            for c in sh.iter("{%s}c" % NS["m"]):
                col, row = re.match(r"([A-Z]+)(\d+)", c.get("r")).groups()
                ci = 0
                for ch in col:
                    ci = ci * 26 + (ord(ch) - 64)
                if c.get("t") == "inlineStr":
                    v = c.find("m:is/m:t", NS).text
                else:
                    v = float(c.find("m:v", NS).text)
                cells[(int(row) - 1, ci - 1)] = v
            out[name] = cells
    return names, out


def _fake(cfg, seed=0):
    rng = np.random.default_rng(seed)
    n, ch = cfg.npix, cfg.chanum
    res = {"acf": rng.normal(size=(n, ch)), "var": rng.uniform(1e-6, 1e-4, (n, ch)),
           "fitres": rng.uniform(0.1, 2, (n, 11)).astype(np.float32), "chi2": rng.uniform(0.5, 2, n).astype(np.float32),
           "fitted": (rng.random(n) > 0.3).astype(np.int32), "blocked_ok": np.ones(n, np.int32)}
    res["acf"][2, 5] = np.nan
    return res


@pytest.mark.parametrize("cfx", [0, 1])
def test_workbook_layout(tmp_path, cfx):
    cfg = engine.FCSConfig(width=5, height=4, frames=3000, cfx=cfx, background=100)
    res = _fake(cfg)
    p = tmp_path / "r.xlsx"
    xlsx.write_results(str(p), cfg, res,
                       diffusion_law={"table": [[0.1, 1.2, 0.04], [0.3, 1.1, 0.02]], "line": (0.05, 0.9),
                                      "fit_range": (1, 2)})
    names, s = read_xlsx(p)
    assert names == xlsx.SHEETS and names[3] == "ACF1" and names[13] == "CCFs" and names[27] == "N&B"
    assert all(len(n) <= 31 for n in names)
    lag, samp = engine.lag_tables(16, 8)
    assert s["lagtime"][(0, 1)] == "Lagtime" and s["lagtime"][(1 + 20, 1)] == pytest.approx(lag[20] * 1e-3)
    assert s["lagtime"][(1 + 40, 2)] == samp[40]
    acf, sd, fp = ("CCFs", "SD (CCF)", "Fit Parameters (CCF)") if cfx else ("ACF1", "SD (ACF1)", "Fit Parameters (ACF1)")
    w = cfg.out_w
    # pixel (x, y) in column x + y * width, channel i in row i + 1
    x, y, i = 2, 1, 7
    assert s[acf][(0, x + y * w)] == f"({x}, {y})"
    assert s[acf][(i + 1, x + y * w)] == pytest.approx(res["acf"][x + y * w, i])
    assert s[sd][(i + 1, x + y * w)] == pytest.approx(np.sqrt(res["var"][x + y * w, i]))
    assert (6, 2) not in s[acf]                                 # NaN -> empty cell
    assert s[fp][(0, 0)] == "Parameter" and s[fp][(1, 0)] == "fitted" and s[fp][(3, 0)] == "D"
    c = 3 + 2 * w
    assert s[fp][(1, c + 1)] == ("true" if res["fitted"][c] else "false")
    assert s[fp][(3, c + 1)] == pytest.approx(float(res["fitres"][c, 1]))
    assert s[fp][(13, c + 1)] == pytest.approx(float(res["chi2"][c]))   # reduced chi^2 row
    d = s["Diffusion Law"]
    assert d[(1, 1)] == pytest.approx(0.1 / 1.2) and d[(1, 3)] == pytest.approx(0.05) and d[(1, 6)] == 2
    assert d[(2, 2)] == pytest.approx(0.3 / 1.1 ** 2 * np.sqrt(0.02))
    assert s["Panel Parameters"][(9, 1)] == "16" and s["Panel Parameters"][(8 - 1, 1)] == str(cfx)


@pytest.mark.gpu
def test_plan_results_roundtrip(tmp_path):
    from tests.synth import brownian_stack
    st = brownian_stack(6, 5, 4000, seed=3, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(width=6, height=5, frames=4000, background=100)
    res = engine.run_host(st, cfg)
    p = tmp_path / "plan.xlsx"
    xlsx.write_results(str(p), cfg, res)
    _, s = read_xlsx(p)
    for c in range(cfg.npix):
        for i in (1, 10, 40):
            if np.isfinite(res["acf"][c, i]):
                assert s["ACF1"][(i + 1, c)] == res["acf"][c, i]
        assert s["Fit Parameters (ACF1)"][(2, c + 1)] == float(res["fitres"][c, 0])


def test_fit_function_sheets(tmp_path):
    """Fit functions and residuals: the model at the fitted parameters over
    the fit range, (acf - fit) / sd there, 0 elsewhere and for pixels
    without a fit (java:10383-10397)."""
    from imaging_fcs_1_52_gb300 import model
    cfg = engine.FCSConfig(width=5, height=4, frames=3000, background=100, fitstart=2, fitend=50)
    rng = np.random.default_rng(1)
    n, ch = cfg.npix, cfg.chanum
    fitres = np.zeros((n, 11), np.float32)
    fitres[:, 0] = rng.uniform(1, 3, n)
    fitres[:, 1] = rng.uniform(0.5, 3, n) * 1e-12
    lag, _ = engine.lag_tables(16, 8)
    truth = model.fcs_model(fitres.astype(float), cfg.cst, lag * 1e-3)
    res = {"acf": truth + rng.normal(0, 1e-3, (n, ch)), "var": np.full((n, ch), 4e-6), "fitres": fitres,
           "chi2": np.ones(n, np.float32), "fitted": (np.arange(n) % 3 != 1).astype(np.int32)}
    p = tmp_path / "f.xlsx"
    xlsx.write_results(str(p), cfg, res)
    _, s = read_xlsx(p)
    fs, rs = s["Fit functions (ACF1)"], s["Residuals (ACF1)"]
    assert fs[(0, 7)] == "(2, 1)" and rs[(0, 7)] == "(2, 1)"
    for c in range(n):
        for i in (1, 2, 30, 50, 51, 72):
            if res["fitted"][c] and 2 <= i <= 50:
                assert fs[(i + 1, c)] == pytest.approx(truth[c, i], rel=1e-12)
                assert rs[(i + 1, c)] == pytest.approx((res["acf"][c, i] - truth[c, i]) / 2e-3, rel=1e-9)
            else:
                assert fs[(i + 1, c)] == 0 and rs[(i + 1, c)] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("gls", [False, True])
def test_fit_curves_reproduce_gpu_chi2(gls):
    """The workbook's residuals of a GPU fit give back the fit's reduced
    chi^2 (java:10403-10406 OLS, 10712-10715 GLS): sum of squared weighted
    residuals over the fit's degrees of freedom."""
    from imaging_fcs_1_52_gb300 import model
    from tests.synth import brownian_stack
    st = brownian_stack(8, 6, 20000, seed=7, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(width=8, height=6, frames=20000, background=100, gls=gls)
    out = engine.run_host(st, cfg)
    lag, _ = engine.lag_tables(cfg.p, cfg.q)
    fit, res = model.fit_curves(out["acf"], out["fitres"], out["fitted"], cfg.cst, lag * cfg.frametime,
                                var=out["var"], covmats=out.get("covmats"), gls=gls, fitstart=1,
                                fitend=cfg.chanum - 1)
    k = 3
    ok = out["fitted"].astype(bool)
    assert ok.sum() >= cfg.npix // 2
    dof = (cfg.chanum - k - 1) if gls else ((cfg.chanum - 1 - 1) - k - 1)
    chi2 = (res[:, 1:] ** 2).sum(axis=1) / dof
    np.testing.assert_allclose(chi2[ok], out["chi2"][ok], rtol=2e-3)


def test_nb_sheet(tmp_path):
    """N&B sheet (java:4999-5017): number and brightness from the lag-1 mean
    and covariance (java:7828-7834), minus the background covariance."""
    cfg = engine.FCSConfig(width=4, height=3, frames=3000)
    rng = np.random.default_rng(2)
    n = cfg.npix
    res = {"nb_mean": rng.uniform(5, 50, n), "nb_cov": rng.uniform(1, 20, n)}
    cov0 = rng.uniform(0, 0.5, (cfg.out_h, cfg.out_w))
    p = tmp_path / "nb.xlsx"
    xlsx.write_results(str(p), cfg, res, nb_background_covariance=cov0)
    _, s = read_xlsx(p)
    nb = s["N&B"]
    assert nb[(1, 0)] == "Number" and nb[(2, 0)] == "Brightness" and nb[(4, 0)] == "Epsilon (corrected)"
    for c in range(n):
        x, y = c % cfg.out_w, c // cfg.out_w
        d = res["nb_cov"][c] - cov0[y, x]
        assert nb[(0, c + 2)] == f"({x}, {y})"
        assert nb[(1, c + 2)] == pytest.approx(res["nb_mean"][c] ** 2 / d, rel=1e-14)
        assert nb[(2, c + 2)] == pytest.approx(d / res["nb_mean"][c], rel=1e-14)
        assert (3, c + 2) not in nb
    # a cross-correlation has no N&B
    ccf = engine.FCSConfig(width=4, height=3, frames=3000, cfx=1)
    xlsx.write_results(str(p), ccf, {"nb_mean": res["nb_mean"][:ccf.npix], "nb_cov": res["nb_cov"][:ccf.npix]})
    _, s = read_xlsx(p)
    assert not s["N&B"]
