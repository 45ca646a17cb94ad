"""Results writer in the plugin's .xlsx layout (Imaging_FCS_1_52.java:4419-5020,
the Apache POI workbook of "Save results").

The workbook has the plugin's sheets in the plugin's order; this engine fills
the ones it computes:

* "Panel Parameters": name / value rows (java:4513-4683) for the settings a
  plan has (image size, frame range, frame time, binning, CF distance,
  correlator P and Q, background, bleach correction, polynomial order);
* "lagtime": S/N, lag time, bin width per channel (java:4685-4694);
* "ACF1" / "SD (ACF1)" for an autocorrelation, "CCFs" / "SD (CCF)" for a
  spatial cross-correlation (the plugin's acf[0] / acf[2]): a header row of
  "(w, h)" labels, then one row per channel, pixel (w, h) in column
  w + h * width (java:4755-4812);
* "Fit Parameters (ACF1)" / "(CCF)": "Parameter" / "fitted" rows, then
  N, D, vx, vy, G, F2, D2, F3, D3, Ftrip, Ttrip, reduced chi^2, blocked
  and valid-pixel rows, pixel (w, h) in column w + h * width + 1
  (java:4816-4862);
* "Diffusion Law": Aeff, time Aeff/D, its SD, then intercept, slope and
  the fit range in the first data row (java:4869-4887, fitDiffLaw
  8207-8210);
* "PSF": the PSF calibration's rows (label, mean D, SD per binning) per PSF
  size, side by side.

* "Fit functions (ACF1)" / "Residuals (ACF1)" (or "(CCF)"): a fitted
  pixel's model curve at the fit's lags and its residuals weighted as the
  fit saw them, 0 for pixels without a fit (java:10383-10397, 10701-10710;
  `model.fit_curves`), laid out as the ACF sheet.

* "N&B": number and brightness of every pixel from the lag-1 monitor and
  covariance of an autocorrelation (the plugin's GPU "G1" mode,
  java:7828-7834): B = (cov - cov0) / mean, N = mean^2 / (cov - cov0), cov0
  the background file's covariance image (0 without one); the "corrected"
  rows, which that mode leaves unset, stay empty (java:4999-5017).

Sheets the engine has no data for (MSD, dCCF, maps) are present and empty, so that readers that address sheets by name or
position find them.  Excel caps sheet names at 31 characters; the plugin's
"Reconstruction Control Parameters" (33) is cut to 31.  Plain OOXML from the
standard library (zipfile); numbers as numbers, NaN as an empty cell.
"""
from __future__ import annotations

import functools
import math
import zipfile
from xml.sax.saxutils import escape

import numpy as np

SHEETS = [
    "Panel Parameters", "Threshold Settings", "lagtime",
    "ACF1", "SD (ACF1)", "Fit functions (ACF1)", "Residuals (ACF1)", "Fit Parameters (ACF1)",
    "ACF2", "SD (ACF2)", "Fit functions (ACF2)", "Residuals (ACF2)", "Fit Parameters (ACF2)",
    "CCFs", "SD (CCF)", "Fit functions (CCF)", "Residuals (CCF)", "Fit Parameters (CCF)",
    "Diffusion Law", "DiffLaw Map Data", "DiffLaw Map SD", "DiffLaw Map Fit",
    "PSF", "MSD of ACF1", "MSD of ACF2", "MSD of CCF", "dCCF", "N&B",
    "Reconstruction Control Parameters"[:31],
]

PARAM_NAMES = ["N", "D", "vx", "vy", "G", "F2", "D2", "F3", "D3", "Ftrip", "Ttrip"]


@functools.lru_cache(maxsize=None)
def _col(c: int) -> str:
    s = ""
    c += 1
    while c:
        c, r = divmod(c - 1, 26)
        s = chr(65 + r) + s
    return s


def _cell(r: int, c: int, v) -> str:
    ref = f"{_col(c)}{r + 1}"
    if v is None:
        return ""
    if isinstance(v, (bool, np.bool_)):
        v = "true" if v else "false"
    if isinstance(v, str):
        return f'<c r="{ref}" t="inlineStr"><is><t>{escape(v)}</t></is></c>'
    x = float(v)
    if not math.isfinite(x):
        return ""
    return f'<c r="{ref}"><v>{repr(x)}</v></c>'


def _block_row(r: int, c0: int, values) -> str:
    """One row of a dense numeric block: cells c0, c0+1, ... (non-finite
    values are left empty)."""
    row = str(r + 1)
    return "".join(f'<c r="{_col(c0 + j)}{row}"><v>{x!r}</v></c>'
                   for j, x in enumerate(values) if math.isfinite(x))


def _sheet_xml(rows: dict, blocks: list) -> str:
    """rows: {row: {col: value}}; blocks: (r0, c0, 2-D float array) placed
    with its element [i][j] at row r0 + i, column c0 + j.  Cells of a row
    are written in column order."""
    out = ['<?xml version="1.0" encoding="UTF-8" standalone="yes"?>',
           '<worksheet xmlns="http://schemas.openxmlformats.org/spreadsheetml/2006/main"><sheetData>']
    by_row: dict = {}
    for r0, c0, a in blocks:
        for i in range(a.shape[0]):
            by_row.setdefault(r0 + i, []).append((c0, a[i]))
    for r in sorted(set(rows) | set(by_row)):
        segs = [(c, _cell(r, c, v)) for c, v in rows.get(r, {}).items()]
        segs += [(c0, _block_row(r, c0, vals.tolist())) for c0, vals in by_row.get(r, [])]
        segs.sort(key=lambda t: t[0])
        out.append(f'<row r="{r + 1}">{"".join(t[1] for t in segs)}</row>')
    out.append("</sheetData></worksheet>")
    return "".join(out)


class Workbook:
    """Cells by sheet name, row, column; written as one .xlsx file."""

    def __init__(self):
        self.cells = {name: {} for name in SHEETS}
        self.blocks = {name: [] for name in SHEETS}

    def set(self, sheet: str, r: int, c: int, v):
        self.cells[sheet].setdefault(r, {})[c] = v

    def set_block(self, sheet: str, r0: int, c0: int, values):
        """Numbers values[i][j] at row r0 + i, column c0 + j (NaN: empty)."""
        self.blocks[sheet].append((r0, c0, np.asarray(values, np.float64)))

    def save(self, path: str):
        ns = "http://schemas.openxmlformats.org/spreadsheetml/2006/main"
        rel = "http://schemas.openxmlformats.org/officeDocument/2006/relationships"
        n = len(SHEETS)
        ct = ['<?xml version="1.0" encoding="UTF-8" standalone="yes"?>',
              '<Types xmlns="http://schemas.openxmlformats.org/package/2006/content-types">',
              '<Default Extension="rels" ContentType="application/vnd.openxmlformats-package.relationships+xml"/>',
              '<Default Extension="xml" ContentType="application/xml"/>',
              '<Override PartName="/xl/workbook.xml" '
              'ContentType="application/vnd.openxmlformats-officedocument.spreadsheetml.sheet.main+xml"/>']
        ct += [f'<Override PartName="/xl/worksheets/sheet{i + 1}.xml" '
               'ContentType="application/vnd.openxmlformats-officedocument.spreadsheetml.worksheet+xml"/>'
               for i in range(n)]
        ct.append("</Types>")
        rels = ('<?xml version="1.0" encoding="UTF-8" standalone="yes"?>'
                '<Relationships xmlns="http://schemas.openxmlformats.org/package/2006/relationships">'
                f'<Relationship Id="rId1" Type="{rel}/officeDocument" Target="xl/workbook.xml"/>'
                "</Relationships>")
        wb = ['<?xml version="1.0" encoding="UTF-8" standalone="yes"?>',
              f'<workbook xmlns="{ns}" xmlns:r="{rel}"><sheets>']
        wb += [f'<sheet name="{escape(name, {chr(34): "&quot;"})}" sheetId="{i + 1}" r:id="rId{i + 1}"/>'
               for i, name in enumerate(SHEETS)]
        wb.append("</sheets></workbook>")
        wrels = ['<?xml version="1.0" encoding="UTF-8" standalone="yes"?>',
                 '<Relationships xmlns="http://schemas.openxmlformats.org/package/2006/relationships">']
        wrels += [f'<Relationship Id="rId{i + 1}" Type="{rel}/worksheet" Target="worksheets/sheet{i + 1}.xml"/>'
                  for i in range(n)]
        wrels.append("</Relationships>")
        with zipfile.ZipFile(path, "w", zipfile.ZIP_DEFLATED, compresslevel=1) as z:
            z.writestr("[Content_Types].xml", "".join(ct))
            z.writestr("_rels/.rels", rels)
            z.writestr("xl/workbook.xml", "".join(wb))
            z.writestr("xl/_rels/workbook.xml.rels", "".join(wrels))
            for i, name in enumerate(SHEETS):
                z.writestr(f"xl/worksheets/sheet{i + 1}.xml", _sheet_xml(self.cells[name], self.blocks[name]))


def _bleach_name(cfg) -> str:
    from . import _lib
    return {_lib.BLEACH_NONE: "none", _lib.BLEACH_SINGLE_EXP: "Single Exp",
            _lib.BLEACH_DOUBLE_EXP: "Double Exp", _lib.BLEACH_POLYNOMIAL: "Polynomial"}.get(cfg.bleach, "")


def nb_maps(nb_mean, nb_cov, background_covariance=None):
    """Number and brightness per pixel from the lag-1 mean and covariance
    (java:7828-7834): B = (cov - cov0) / mean, N = mean^2 / (cov - cov0)."""
    m = np.asarray(nb_mean, float)
    c = np.asarray(nb_cov, float) - (0.0 if background_covariance is None else
                                     np.asarray(background_covariance, float).reshape(m.shape))
    with np.errstate(divide="ignore", invalid="ignore"):
        return m * m / c, c / m


def write_results(path: str, cfg, results: dict, *, lagtime=None, samp=None, diffusion_law=None,
                  psf=None, nb_background_covariance=None) -> None:
    """Write a plan's results (engine.Plan.execute_host outputs) in the plugin's
    workbook layout.  cfg: the engine.FCSConfig; results: acf, sd or var,
    fitres, chi2, fitted, blocked_ok (any may be missing); lagtime, samp:
    per-channel lag time (s) and bin width (default: the lag tables of
    cfg); diffusion_law: dict with "table" (n_bin x 3: Aeff um^2, mean D
    um^2/s, var D) and optionally "line" (intercept, slope) and "fit_range";
    psf: array [psf][3][n_bin] from imfcs_psf_calibration;
    nb_background_covariance: the background file's covariance image
    [out_h][out_w] for the N&B sheet (imfcs_background_stats)."""
    wb = Workbook()
    w, h = cfg.out_w, cfg.out_h
    # Panel Parameters: the plugin's first rows, values where a plan has them
    panel = [("Image width", cfg.width), ("Image height", cfg.height), ("First frame", cfg.first + 1),
             ("Last frame", cfg.first + cfg.num), ("Frame time", cfg.frametime), ("Binning X", cfg.binx),
             ("Binning Y", cfg.biny), ("CF X distance", cfg.cfx), ("CF Y distance", cfg.cfy),
             ("Correlator P", cfg.p), ("Correlator Q", cfg.q), ("Fit model", "ITIR-FCS (2D)"),
             ("FCCS Display", ""), ("PixelSize", ""), ("Overlap", str(cfg.pixbinx < cfg.binx).lower()),
             ("Magnification", ""), ("NA", ""), ("Em Lambda", ""), ("Em Lambda2", ""), ("Sigma", ""),
             ("SigmaZ", ""), ("Sigma2", ""), ("SigmaZ2", ""), ("Background", cfg.background),
             ("Background2", cfg.background), ("Background File", ""), ("Bleach Correction", _bleach_name(cfg)),
             ("Sliding Window Length", ""), ("Polynomial Order", cfg.poly_order), ("Filter", ""),
             ("filterUL", ""), ("filterLL", ""), ("Threshold", ""), ("Fit", str(bool(cfg.do_fit)).lower())]
    for r, (k, v) in enumerate(panel):
        wb.set("Panel Parameters", r, 0, k)
        wb.set("Panel Parameters", r, 1, str(v))
    # lag times
    if lagtime is None or samp is None:
        from .engine import lag_tables
        lag, samp = lag_tables(cfg.p, cfg.q)
        lagtime = lag * cfg.frametime
    ch = cfg.chanum
    wb.set("lagtime", 0, 0, "S/N")
    wb.set("lagtime", 0, 1, "Lagtime")
    wb.set("lagtime", 0, 2, "Bin width")
    for i in range(ch):
        wb.set("lagtime", i + 1, 0, i)
        wb.set("lagtime", i + 1, 1, float(lagtime[i]))
        wb.set("lagtime", i + 1, 2, float(samp[i]))
    # correlation and SD: acf[0] (ACF1) or acf[2] (CCFs)
    ccf = bool(cfg.cfx or cfg.cfy)
    acf_sheet, sd_sheet, fit_sheet = (("CCFs", "SD (CCF)", "Fit Parameters (CCF)") if ccf else
                                      ("ACF1", "SD (ACF1)", "Fit Parameters (ACF1)"))
    label = {}
    for y in range(h):
        for x in range(w):
            label[x + y * w] = f"({x}, {y})"
    sd = results.get("sd")
    if sd is None and results.get("var") is not None:
        sd = np.sqrt(results["var"])
    for name, data, sheet in (("acf", results.get("acf"), acf_sheet), ("sd", sd, sd_sheet)):
        if data is None:
            continue
        for c, lab in label.items():
            wb.set(sheet, 0, c, lab)
        wb.set_block(sheet, 1, 0, np.asarray(data, float)[:w * h, :ch].T)
    # fit functions and residuals of the fitted pixels
    fr = results.get("fitres")
    acf = results.get("acf")
    var = results.get("var")
    if var is None and sd is not None:
        var = np.asarray(sd, float) ** 2
    if fr is not None and acf is not None and results.get("fitted") is not None and \
            (var is not None if not cfg.gls else results.get("covmats") is not None):
        from .model import fit_curves
        fs = max(int(cfg.fitstart), 1)
        fe = ch - 1 if cfg.fitend is None or cfg.fitend >= ch or cfg.fitend < fs else int(cfg.fitend)
        fit, res = fit_curves(acf, fr, results["fitted"], cfg.cst, lagtime, var=var,
                              covmats=results.get("covmats"), gls=bool(cfg.gls), fitstart=fs, fitend=fe)
        tag = "CCF" if ccf else "ACF1"
        for data, sheet in ((fit, f"Fit functions ({tag})"), (res, f"Residuals ({tag})")):
            for c, lab in label.items():
                wb.set(sheet, 0, c, lab)
            wb.set_block(sheet, 1, 0, data[:w * h, :ch].T)
    # fit parameters
    if fr is not None:
        wb.set(fit_sheet, 0, 0, "Parameter")
        wb.set(fit_sheet, 1, 0, "fitted")
        names = PARAM_NAMES + ["reduced Chi2", "blocked", "valid pixels"]
        for q, nm in enumerate(names):
            wb.set(fit_sheet, q + 2, 0, nm)
        fitted = results.get("fitted")
        chi2 = results.get("chi2")
        blocked = results.get("blocked_ok")
        npx = w * h
        for c, lab in label.items():
            wb.set(fit_sheet, 0, c + 1, lab)
            wb.set(fit_sheet, 1, c + 1, bool(fitted[c]) if fitted is not None else None)
        wb.set_block(fit_sheet, 2, 1, np.asarray(fr, float)[:npx, :len(PARAM_NAMES)].T)
        for q, extra in enumerate((chi2, blocked, fitted)):
            if extra is not None:
                wb.set_block(fit_sheet, len(PARAM_NAMES) + 2 + q, 1, np.asarray(extra, float)[None, :npx])
    # N&B of an autocorrelation
    if not ccf and results.get("nb_mean") is not None and results.get("nb_cov") is not None:
        num, bright = nb_maps(results["nb_mean"], results["nb_cov"], nb_background_covariance)
        for r, nm in enumerate((" ", "Number", "Brightness", "Num (corrected)", "Epsilon (corrected)")):
            wb.set("N&B", r, 0, nm)
        for c, lab in label.items():
            wb.set("N&B", 0, c + 2, lab)
            wb.set("N&B", 1, c + 2, float(num[c]))
            wb.set("N&B", 2, c + 2, float(bright[c]))
    # diffusion law
    if diffusion_law is not None:
        t = np.asarray(diffusion_law["table"], float)
        for c, nm in enumerate(("Aeff", "Time", "SD", "intercept", "slope", "fit start", "fit end")):
            wb.set("Diffusion Law", 0, c, nm)
        for i in range(len(t)):
            aeff, d, v = t[i]
            wb.set("Diffusion Law", i + 1, 0, aeff)
            wb.set("Diffusion Law", i + 1, 1, aeff / d)
            wb.set("Diffusion Law", i + 1, 2, aeff / (d * d) * math.sqrt(v) if v >= 0 else float("nan"))
        if diffusion_law.get("line") is not None:
            wb.set("Diffusion Law", 1, 3, float(diffusion_law["line"][0]))
            wb.set("Diffusion Law", 1, 4, float(diffusion_law["line"][1]))
        if diffusion_law.get("fit_range") is not None:
            wb.set("Diffusion Law", 1, 5, float(diffusion_law["fit_range"][0]))
            wb.set("Diffusion Law", 1, 6, float(diffusion_law["fit_range"][1]))
    # PSF calibration: per PSF size, three columns (bin label, mean D, SD)
    if psf is not None:
        p = np.asarray(psf, float)
        for k in range(p.shape[0]):
            for j, nm in enumerate(("bin", "D", "SD")):
                wb.set("PSF", 0, 3 * k + j, f"{nm} (PSF {k + 1})")
                for b in range(p.shape[2]):
                    wb.set("PSF", b + 1, 3 * k + j, float(p[k, j, b]))
    wb.save(path)
