"""The Python mirror of the plugin's gpufitImFCS.GpufitImFCS class
(imaging_fcs_1_52_gb300.gpufit_imfcs): its types and defaults against
GpufitImFCS.java, its error behaviour, and -- on a GPU -- that each native
it wraps returns what the C ABI returns for the same arguments."""
import ctypes as C

import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib
from imaging_fcs_1_52_gb300.gpufit_imfcs import (ACFParameters, Estimator, FitModel, FitResult, FitState,
                                                 GpufitImFCS, Model)


def _cuda() -> bool:
    import torch
    return torch.cuda.is_available()


def test_types_follow_the_java_class():
    # Model enum (GpufitImFCS.java:883): id and parameter count
    assert (Model.GAUSS_2D.id, Model.GAUSS_2D.numberParameters) == (1, 5)
    assert (Model.ACF_1D.id, Model.ACF_1D.numberParameters) == (2, 20)
    assert (Model.LINEAR_1D.id, Model.LINEAR_1D.numberParameters) == (3, 11)
    assert int(Estimator.LSE) == 0 and int(FitState.CONVERGED) == 0 and int(FitState.MAX_ITERATIONS) == 1
    # FitModel defaults (GpufitImFCS.java:707-708)
    fm = FitModel(4, 72, True, Model.ACF_1D, parametersToFit=[True, True, False] + [False] * 17,
                  userInfoSize=72 * 4)
    assert fm.tolerance == pytest.approx(1e-4) and fm.maxNumberIterations == 25
    assert fm.data.size == 4 * 72 and fm.weights.size == 4 * 72 and fm.initialParameters.size == 4 * 20
    assert list(fm.parametersToFit[:4]) == [1, 1, 0, 0] and fm.userInfo.size == 72
    assert FitModel(2, 10, False, Model.LINEAR_1D).weights is None
    # FitResult sizes and the compatibility check
    fr = FitResult(4, 20)
    assert fr.parameters.size == 80 and fr.states.size == 4
    fr.isCompatible(4, 20)
    with pytest.raises(RuntimeError, match="parameters"):
        fr.isCompatible(5, 20)


def test_errors_without_a_device():
    if _cuda():
        pytest.skip("a device is present")
    assert GpufitImFCS.isCudaAvailable() is False
    fm = FitModel(2, 72, True, Model.ACF_1D, userInfoSize=72 * 4)
    with pytest.raises(RuntimeError, match="status = "):
        GpufitImFCS.fit(fm)
    p = ACFParameters(win_star=4, hin_star=4, w_temp=4, h_temp=4, binningX=1, binningY=1, pixbinX=1,
                      pixbinY=1, firstframe=1, lastframe=10)
    with pytest.raises(RuntimeError):
        GpufitImFCS.calcBinning(np.zeros((10, 4, 4)), np.zeros((10, 4, 4), np.float32), p)


def test_output_arrays_must_be_float32():
    p = ACFParameters(win_star=4, hin_star=4, w_temp=4, h_temp=4, binningX=1, binningY=1, pixbinX=1,
                      pixbinY=1, firstframe=1, lastframe=10)
    with pytest.raises(ValueError, match="float32"):
        GpufitImFCS.calcBinning(np.zeros((10, 4, 4)), np.zeros((10, 4, 4)), p)


@pytest.mark.gpu
def test_fit_matches_the_c_abi():
    """GpufitImFCS.fit (ACF_1D, weighted, N, D, G free) against the same
    call of imfcs_fit: same parameters, states, chi-squares, iterations."""
    from tests.test_gpu_fit import _acf_curves
    n, npts = 24, 72
    data, var, lagtime, cst = _acf_curves(n, seed=5)
    fm = FitModel(n, npts, True, Model.ACF_1D, tolerance=1e-16, maxNumberIterations=2000,
                  parametersToFit=[i in (0, 1, 4) for i in range(20)], userInfoSize=npts * 4)
    fm.data[:] = data[:, 1:].astype(np.float32).ravel()
    fm.weights[:] = (1.0 / var[:, 1:]).astype(np.float32).ravel()
    init = fm.initialParameters.reshape(n, 20)
    init[:, 0], init[:, 1], init[:, 11:20] = 1.0, 1e-12, cst
    fm.userInfo[:] = lagtime[1:]
    res = GpufitImFCS.fit(fm)
    L = _lib.load()
    outp = np.zeros(n * 20, np.float32)
    st = np.zeros(n, np.int32)
    chi = np.zeros(n, np.float32)
    it = np.zeros(n, np.int32)
    rc = L.imfcs_fit(n, npts, fm.data.ctypes.data, fm.weights.ctypes.data, 2, fm.initialParameters.ctypes.data,
                     C.c_float(1e-16), 2000, 0, fm.parametersToFit.ctypes.data, 0, fm.userInfo.nbytes,
                     fm.userInfo.ctypes.data, outp.ctypes.data, st.ctypes.data, chi.ctypes.data, it.ctypes.data)
    assert rc == 0, _lib.last_error()
    np.testing.assert_array_equal(res.parameters, outp)
    np.testing.assert_array_equal(res.states, st)
    np.testing.assert_array_equal(res.chiSquares, chi)
    np.testing.assert_array_equal(res.numberIterations, it)
    assert (res.states == FitState.CONVERGED).mean() >= 0.9 and res.fitDuration > 0
    # a FitResult of the wrong size is refused before the native runs
    with pytest.raises(RuntimeError, match="size"):
        GpufitImFCS.fit(fm, FitResult(n + 1, 20))


@pytest.mark.gpu
def test_calc_binning_bleach_average_and_acf_match_the_c_abi():
    from tests.synth import brownian_stack
    assert GpufitImFCS.isCudaAvailable()
    v = GpufitImFCS.getCudaVersion()
    assert v.runtime.startswith("13.") and v.driver != "0.0"
    raw = brownian_stack(9, 8, 4000, seed=31, density=2.0, cps=3e4).astype(np.float32) - 100
    bx = by = 2
    wt, ht = 9 - bx + 1, 8 - by + 1
    p = ACFParameters(width=3, height=3, win_star=9, hin_star=8, w_temp=wt, h_temp=ht, pixbinX=bx, pixbinY=by,
                      binningX=bx, binningY=by, firstframe=1, lastframe=4000, framediff=4000, cfXDistance=0,
                      cfYDistance=0, correlatorp=16, correlatorq=8, frametime=1e-3, background=100, chanum=73,
                      isNBcalculation=0, bleachcorr_gpu=0, bleachcorr_order=0, nopit=1000, ave=4)
    assert GpufitImFCS.isBinningMemorySufficient(p) and GpufitImFCS.isACFmemorySufficient(p)
    binned = np.zeros((4000, ht, wt), np.float32)
    GpufitImFCS.calcBinning(raw, binned, p)
    np.testing.assert_array_equal(binned, sum(raw[:, j:j + ht, i:i + wt] for i in range(bx) for j in range(by)))
    avg = np.zeros((ht, wt, 1000), np.float32)
    GpufitImFCS.calcDataBleachCorrection(binned, avg, p)
    want = np.zeros_like(avg)
    L = _lib.load()
    assert L.imfcs_calc_data_bleach_correction(binned.ctypes.data, want.ctypes.data, C.byref(p)) == 0
    np.testing.assert_array_equal(avg, want)
    outs = [np.zeros((73, 3, 3)), np.zeros((73, 3, 3)), np.zeros((3, 3)), np.zeros((3, 3)), np.zeros((2, 3, 3))]
    samp, lag = np.zeros(73), np.zeros(73, np.int32)
    GpufitImFCS.calcACF(binned, *outs, None, samp, lag, p)
    ref = [np.zeros_like(o) for o in outs]
    samp2, lag2 = np.zeros(73), np.zeros(73, np.int32)
    assert L.imfcs_calc_acf(binned.ctypes.data, *[r.ctypes.data for r in ref], None, samp2.ctypes.data,
                            lag2.ctypes.data, C.byref(p)) == 0
    for o, r in zip(outs, ref):
        np.testing.assert_array_equal(o, r)
    np.testing.assert_array_equal(lag, lag2)
    assert np.isfinite(outs[0][1]).all()
    # a native error surfaces as RuntimeError with the library's message
    bad = ACFParameters.from_buffer_copy(p)
    bad.correlatorp = 12
    with pytest.raises(RuntimeError):
        GpufitImFCS.calcACF(binned, *[np.zeros_like(o) for o in outs], None, samp, lag, bad)
