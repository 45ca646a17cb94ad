"""Band-streamed host execution (imfcs_bands_*): a job's output rows split
into bands whose input rows are copied and correlated one band at a time.

CPU: the band split (imfcs_band_window, host arithmetic) against a
restatement of the window geometry -- every output row added exactly once,
every window of a band's rows inside its buffer, the buffer inside the
image.  GPU: bands give the results of the whole-stack execution
(imfcs_plan_execute_host), pixel for pixel."""
import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib, engine

GEOMETRIES = [
    dict(width=12, height=21),                                               # ACF, bin 1
    dict(width=12, height=21, cfy=2),                                        # CCF down
    dict(width=12, height=21, cfx=1, cfy=-1, map_y0=1, out_h=20),            # CCF up (halo above)
    dict(width=13, height=22, binx=2, biny=2),                               # non-overlapping bin 2
    dict(width=13, height=22, binx=2, biny=2, pixbinx=1, pixbiny=1),         # overlapping bin 2
    dict(width=14, height=25, binx=3, biny=3, cfy=-2, map_y0=1, out_h=6),    # bin 3, cfy not a multiple
    dict(width=10, height=17, biny=2, binx=2, cfy=-3, map_y0=2, out_h=5),    # halo above, shifted map
]


def _windows_rows(cfg, oy):
    """Input rows output row oy reads (both windows)."""
    y = (cfg.map_y0 + oy) * cfg.pixbiny
    return y + min(0, cfg.cfy), y + cfg.biny - 1 + max(0, cfg.cfy)


@pytest.mark.parametrize("geo", GEOMETRIES)
@pytest.mark.parametrize("band_rows", [1, 2, 3, 5, 100])
def test_band_split_covers_every_row_once(geo, band_rows):
    cfg = engine.FCSConfig(frames=100, **geo)
    wins = engine.band_windows(cfg, band_rows)
    rows = min(band_rows, cfg.out_h)
    assert len(wins) == -(-cfg.out_h // rows)
    added = []
    for w in wins:
        added += list(range(w["new_row0"], w["new_row0"] + w["new_rows"]))
        assert w["out_row0"] <= w["new_row0"] and w["new_row0"] + w["new_rows"] <= w["out_row0"] + rows
        assert w["in_rows"] == wins[0]["in_rows"]
        # every window of the band's rows lies in its buffer and in the image
        for oy in range(w["out_row0"], w["out_row0"] + rows):
            lo, hi = _windows_rows(cfg, oy)
            assert w["in_row0"] <= lo and hi < w["in_row0"] + w["in_rows"]
            assert lo >= 0 and hi < cfg.height
        assert 0 <= w["in_row0"] and w["in_row0"] + w["in_rows"] <= cfg.height
        # the band's first output row sits at a whole pixel step in its buffer
        assert ((cfg.map_y0 + w["out_row0"]) * cfg.pixbiny - w["in_row0"]) % cfg.pixbiny == 0
    assert added == list(range(cfg.out_h))


def test_band_split_rejects_bad_arguments():
    cfg = engine.FCSConfig(width=8, height=8, frames=100)
    with pytest.raises(_lib.ImfcsError):
        engine.band_windows(cfg, 0)
    bad = engine.FCSConfig(width=8, height=8, frames=100, out_h=9)
    with pytest.raises(_lib.ImfcsError):
        engine.band_windows(bad, 2)


def _compare(whole, banded, names):
    for n in names:
        a, b = whole[n], banded[n]
        if a.dtype.kind == "f":
            np.testing.assert_array_equal(np.isnan(a), np.isnan(b), err_msg=n)
            np.testing.assert_allclose(b[~np.isnan(b)], a[~np.isnan(a)], rtol=1e-6, atol=0, err_msg=n)
        else:
            np.testing.assert_array_equal(b, a, err_msg=n)


GPU_CASES = [
    ("acf-exp", dict(width=12, height=21, bleach=_lib.BLEACH_SINGLE_EXP), 4),
    ("ccf-up-poly", dict(width=12, height=21, cfx=1, cfy=-1, map_y0=1, out_h=20, bleach=_lib.BLEACH_POLYNOMIAL), 6),
    ("bin3-cfy-2", dict(width=14, height=25, binx=3, biny=3, cfy=-2, map_y0=1, out_h=6), 2),
    ("overlap-bin2-first", dict(width=13, height=22, binx=2, biny=2, pixbinx=1, pixbiny=1, first=500), 7),
    ("gls-bayes", dict(width=8, height=10, gls=True, bayes=True), 3),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,geo,band_rows", GPU_CASES, ids=[c[0] for c in GPU_CASES])
def test_bands_match_whole_stack(name, geo, band_rows):
    from tests.synth import brownian_stack
    st = brownian_stack(geo["width"], geo["height"], 6000, seed=11, density=2.0, cps=3e4, tau_bleach=3.0)
    cfg = engine.FCSConfig(frames=6000, background=100, **geo)
    whole = engine.run_host(st, cfg)
    bands = engine.Bands(cfg, band_rows=band_rows)
    g = bands.geometry()
    assert g["band_rows"] == min(band_rows, cfg.out_h) and g["bands"] == -(-cfg.out_h // g["band_rows"])
    out = bands.execute_host(st)
    _compare(whole, out, engine.output_names(cfg))
    # a second execution of the same bands object gives the same results
    again = bands.execute_host(st)
    _compare(out, again, engine.output_names(cfg))
    bands.close()


@pytest.mark.gpu
def test_bands_sized_from_a_device_budget():
    """A budget below the whole job's footprint gives several bands whose
    footprint fits; the results are still the whole stack's."""
    from tests.synth import brownian_stack
    st = brownian_stack(16, 24, 4000, seed=5, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(width=16, height=24, frames=4000, background=100)
    whole_b = engine.Bands(cfg, band_rows=cfg.out_h)
    full = whole_b.geometry()["device_bytes"]
    whole_b.close()
    budget = full // 3
    bands = engine.Bands(cfg, max_device_bytes=budget)
    g = bands.geometry()
    assert g["bands"] >= 3 and g["device_bytes"] <= budget
    out = bands.execute_host(st)
    _compare(engine.run_host(st, cfg), out, engine.output_names(cfg))
    bands.close()
    with pytest.raises(_lib.ImfcsError):
        engine.Bands(cfg, max_device_bytes=1 << 16)


@pytest.mark.gpu
def test_bands_refuse_a_background_image():
    """A background image on the band plan would cover one band's rows only:
    execution is refused."""
    import ctypes as C
    cfg = engine.FCSConfig(width=8, height=8, frames=6000)
    bands = engine.Bands(cfg, band_rows=3)
    rows = engine.band_windows(cfg, 3)[0]["in_rows"]
    bg = np.full((rows, cfg.width), 100.0)
    L = _lib.load()
    _lib.check(L.imfcs_plan_set_background_image(L.imfcs_bands_plan(bands._h), C.c_void_p(bg.ctypes.data)),
               "imfcs_plan_set_background_image")
    with pytest.raises(_lib.ImfcsError, match="background image"):
        bands.execute_host(np.zeros((6000, 8, 8), np.uint16))
    bands.close()


@pytest.mark.gpu
def test_bands_with_a_background_image_match_whole_stack():
    """A per-pixel background image on bands (each band takes its rows)
    gives the whole-stack results with the same image."""
    from tests.synth import brownian_stack
    geo = dict(width=12, height=21, binx=2, biny=2, pixbinx=1, pixbiny=1, cfx=1, cfy=-1, map_y0=1, out_h=18)
    st = brownian_stack(12, 21, 6000, seed=13, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(frames=6000, background=100, **geo)
    bg = np.random.default_rng(3).uniform(95.0, 105.0, (21, 12))
    plan = engine.Plan(cfg)
    plan.set_background_image(bg)
    whole = plan.execute_host(st)
    plan.close()
    bands = engine.Bands(cfg, band_rows=5)
    bands.set_background_image(bg)
    _compare(whole, bands.execute_host(st), engine.output_names(cfg))
    # back to the scalar background
    bands.set_background_image(None)
    _compare(engine.run_host(st, cfg), bands.execute_host(st), engine.output_names(cfg))
    bands.close()


@pytest.mark.parametrize("geo,band_rows", [
    (dict(width=9, height=14, cfy=2), 4),
    (dict(width=9, height=14, cfx=1, cfy=-1, map_y0=1, out_h=13), 3),
    (dict(width=10, height=17, binx=2, biny=2, pixbinx=1, pixbiny=1, cfy=-3, map_y0=3, out_h=12), 5),
    (dict(width=14, height=25, binx=3, biny=3, cfy=-2, map_y0=1, out_h=6), 4),
])
def test_band_decomposition_preserves_every_pixel_on_the_oracle(geo, band_rows):
    """The band split on the CPU, with the oracle as each band's engine:
    every band's sub-stack (its input rows, frames first..first+num-1) under
    the band geometry (map_y0 = the halo's pixel steps, out_h = band rows)
    gives the whole stack's per-pixel results."""
    import oracle
    from tests.synth import brownian_stack
    cfg = engine.FCSConfig(frames=3000, first=200, background=100, **geo)
    st = brownian_stack(cfg.width, cfg.height, 3000, seed=21, density=2.0, cps=3e4)
    kw = dict(out_w=cfg.out_w, map_x0=cfg.map_x0, binx=cfg.binx, biny=cfg.biny, pixbinx=cfg.pixbinx,
              pixbiny=cfg.pixbiny, cfx=cfg.cfx, cfy=cfg.cfy, background=100, p=16, q=7, do_fit=False)
    whole = oracle.run(st, out_h=cfg.out_h, map_y0=cfg.map_y0, first=cfg.first, num=cfg.num, **kw)
    got = {k: np.full_like(whole[k], -7) for k in ("acf", "var", "blocked_ind", "blocked_ok")}
    for w in engine.band_windows(cfg, band_rows):
        rows = min(band_rows, cfg.out_h)
        m = cfg.map_y0 + w["out_row0"] - w["in_row0"] // cfg.pixbiny
        assert w["in_row0"] % cfg.pixbiny == 0 and m >= 0
        sub = st[cfg.first:cfg.first + cfg.num, w["in_row0"]:w["in_row0"] + w["in_rows"]]
        band = oracle.run(sub, out_h=rows, map_y0=m, **kw)
        skip = w["new_row0"] - w["out_row0"]
        for k in got:
            got[k][w["new_row0"] * cfg.out_w:(w["new_row0"] + w["new_rows"]) * cfg.out_w] = \
                band[k][skip * cfg.out_w:(skip + w["new_rows"]) * cfg.out_w]
    for k in got:
        np.testing.assert_array_equal(got[k], whole[k], err_msg=k)


def test_band_split_random_geometries():
    """imfcs_band_window over 300 random valid geometries: rows added once
    each, windows inside the band buffer, buffer inside the image."""
    rng = np.random.default_rng(8)
    checked = 0
    while checked < 300:
        b = int(rng.integers(1, 5))
        over = bool(rng.integers(0, 2))
        step = 1 if over else b
        cfy = int(rng.integers(-4, 5))
        h = int(rng.integers(b + abs(cfy) + 1, 40))
        y0min = -(-max(0, -cfy) // step)                 # first map row whose window stays in the image
        rows_max = (h - 1 - max(0, cfy) - (b - 1)) // step + 1 - y0min
        if rows_max < 1:
            continue
        map_y0 = int(rng.integers(y0min, y0min + rows_max))
        out_h = int(rng.integers(1, rows_max - (map_y0 - y0min) + 1))
        cfg = engine.FCSConfig(width=6, height=h, frames=100, binx=b, biny=b, pixbinx=step, pixbiny=step,
                               cfy=cfy, map_y0=map_y0, out_h=out_h)
        band_rows = int(rng.integers(1, out_h + 2))
        wins = engine.band_windows(cfg, band_rows)
        rows = min(band_rows, out_h)
        added = []
        for w in wins:
            added += range(w["new_row0"], w["new_row0"] + w["new_rows"])
            assert 0 <= w["in_row0"] and w["in_row0"] + w["in_rows"] <= h
            for oy in range(w["out_row0"], w["out_row0"] + rows):
                lo, hi = _windows_rows(cfg, oy)
                assert w["in_row0"] <= lo and hi < w["in_row0"] + w["in_rows"]
        assert added == list(range(out_h))
        checked += 1
