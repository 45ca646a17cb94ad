"""GPU parity of the correlator through the C ABI (imfcs_plan_execute_host)
against the FP64 oracle: blocking index and flag exactly, ACF within
ACF_TOL * |G(lag 1)|, blocked variance within VAR_TOL relative."""
import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib, engine
from tests.helpers import ACF_TOL, VAR_TOL, acf_deviation, run_both
from tests.synth import bleach_stack, brownian_stack

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dim_stack():
    return brownian_stack(8, 8, 4000, seed=3)


@pytest.fixture(scope="module")
def bright_bleached():
    return brownian_stack(8, 8, 4000, seed=5, tau_bleach=2.0, density=3.0, cps=1e5)


@pytest.fixture(scope="module")
def bright_two_rate_bleach():
    return bleach_stack(8, 8, 4000, seed=6, fluct=0.05)


def check_acf(gpu, ref):
    """Blocking index and flag exactly; finiteness per lag exactly (a
    non-finite corrected frame makes exactly the lags whose windows hold it
    non-finite, java:9484-9511); at every finite lag the ACF within ACF_TOL
    of the pixel's |G(lag 1)| and the blocked variance within VAR_TOL (max)
    and 1e-5 (median) relative."""
    np.testing.assert_array_equal(gpu["blocked_ind"], ref["blocked_ind"])
    np.testing.assert_array_equal(gpu["blocked_ok"], ref["blocked_ok"])
    np.testing.assert_array_equal(np.isfinite(gpu["acf"]), np.isfinite(ref["acf"]))
    assert acf_deviation(gpu, ref) <= ACF_TOL
    v_g, v_r = gpu["var"][:, 1:], ref["var"][:, 1:]
    fin = np.isfinite(v_r)
    np.testing.assert_array_equal(np.isfinite(v_g), fin)
    if fin.any():
        rel = np.abs(v_g[fin] - v_r[fin]) / np.abs(v_r[fin])
        assert rel.max() <= VAR_TOL and np.median(rel) <= 1e-5


@pytest.mark.parametrize("kw", [
    {},
    {"q": 6},
    {"q": 4},
    {"q": 3, "cfx": 1, "cfy": 1},
    {"binx": 2, "biny": 2},
    {"binx": 3, "biny": 2, "pixbinx": 1, "pixbiny": 1},
    {"cfx": 1, "cfy": 0},
    {"cfx": 0, "cfy": 2},
    {"cfx": 2, "cfy": 1},
], ids=["acf", "q6", "q4", "q3-ccf11", "bin2", "bin3x2-overlap", "ccf10", "ccf02", "ccf21"])
def test_correlator_no_bleach(dim_stack, kw):
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100, do_fit=False, **kw)
    gpu, ref = run_both(dim_stack, cfg)
    check_acf(gpu, ref)


@pytest.mark.parametrize("order", [1, 2, 4, 8])
def test_correlator_polynomial_bleach(dim_stack, order):
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100, do_fit=False,
                           bleach=_lib.BLEACH_POLYNOMIAL, poly_order=order)
    gpu, ref = run_both(dim_stack, cfg)
    check_acf(gpu, ref)


def test_correlator_single_exponential_bleach(bright_bleached):
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100, do_fit=False,
                           bleach=_lib.BLEACH_SINGLE_EXP)
    gpu, ref = run_both(bright_bleached, cfg)
    check_acf(gpu, ref)


def test_correlator_double_exponential_bleach(bright_two_rate_bleach):
    # a trace dominated by a two-rate bleach (0.4 s and 4 s): both rates are
    # resolved, so the least-squares minimum is unique
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100, do_fit=False,
                           bleach=_lib.BLEACH_DOUBLE_EXP)
    gpu, ref = run_both(bright_two_rate_bleach, cfg)
    check_acf(gpu, ref)


def test_minimum_frames():
    # 2176 frames is the minimum for P=16, Q=8 (java:7315)
    st = brownian_stack(4, 4, 2176, seed=8, density=2.0)
    cfg = engine.FCSConfig(width=4, height=4, frames=2176, background=100, do_fit=False)
    gpu, ref = run_both(st, cfg)
    check_acf(gpu, ref)


def test_frame_range_and_map_offset(dim_stack):
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, first=300, num=3500, background=100, do_fit=False,
                           map_x0=2, map_y0=1, out_w=5, out_h=6)
    gpu, ref = run_both(dim_stack, cfg)
    check_acf(gpu, ref)


def test_nb_outputs(dim_stack):
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100, do_fit=False)
    gpu, ref = run_both(dim_stack, cfg)
    # N&B (agpufitjni.cu:5176-5179): lag-1 direct monitor and covariance
    c = np.array([oracle_nb(dim_stack, p % 8, p // 8) for p in range(64)])
    np.testing.assert_allclose(gpu["nb_mean"], c[:, 0], rtol=1e-6)
    np.testing.assert_allclose(gpu["nb_cov"], c[:, 1], rtol=1e-4, atol=1e-4 * np.abs(c[:, 1]).max())


def oracle_nb(stack, x, y):
    import oracle
    tr = oracle.get_intensity(stack, x, y, bckg=100)[1:]
    d, e = tr[:-1], tr[1:]
    dm, Dm = d.mean(), e.mean()
    return dm, np.mean((d - dm) * (e - Dm))


def test_determinism(dim_stack):
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100, bleach=_lib.BLEACH_POLYNOMIAL,
                           poly_order=3)
    a = engine.run_host(dim_stack, cfg)
    b = engine.run_host(dim_stack, cfg)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
