"""Python mirror of the plugin's JNI class gpufitImFCS.GpufitImFCS
(GpufitImFCS.java), bound to the GB300 library's C ABI.

Same names, argument meaning and error behaviour as the Java class: arrays
are passed in and filled in place, a failed fit raises RuntimeError("status
= ..., message = ...") (GpufitImFCS.java:344-360), the calc* natives raise on
error like the JNI's ThrowNew (agpufitjni.cu:4792-4806, 5795-5830).
"""
from __future__ import annotations

import ctypes as C
import enum
import time
from dataclasses import dataclass

import numpy as np

from . import _lib

ACFParameters = _lib.ACFParameters


class Estimator(enum.IntEnum):
    LSE = 0
    MLE = 1


class FitState(enum.IntEnum):
    CONVERGED = 0
    MAX_ITERATIONS = 1
    SINGULAR_HESSIAN = 2
    NEG_CURVATURE_MLE = 3
    GPU_NOT_READY = 4


class Model(enum.Enum):
    GAUSS_2D = (1, 5)
    ACF_1D = (2, 20)
    LINEAR_1D = (3, 11)

    @property
    def id(self) -> int:
        return self.value[0]

    @property
    def numberParameters(self) -> int:
        return self.value[1]


@dataclass
class CudaVersion:
    runtime: str
    driver: str


class FitModel:
    """GpufitImFCS.FitModel (GpufitImFCS.java:611-669)."""

    def __init__(self, numberFits, numberPoints, withWeights, model: Model, tolerance=None,
                 maxNumberIterations=None, num_valid_coefs=0, parametersToFit=None, estimator=None,
                 userInfoSize=0):
        self.numberFits = numberFits
        self.numberPoints = numberPoints
        self.data = np.zeros(numberFits * numberPoints, np.float32)
        self.weights = np.zeros(numberFits * numberPoints, np.float32) if withWeights else None
        self.model = model
        self.initialParameters = np.zeros(numberFits * model.numberParameters, np.float32)
        self.tolerance = 1e-4 if tolerance is None else float(tolerance)
        self.maxNumberIterations = 25 if maxNumberIterations is None else int(maxNumberIterations)
        self.num_valid_coefs = int(num_valid_coefs)
        if parametersToFit is None:
            self.parametersToFit = np.ones(model.numberParameters, np.int32)
        else:
            self.parametersToFit = np.array([1 if p else 0 for p in parametersToFit], np.int32)
        self.estimator = Estimator.LSE if estimator is None else estimator
        # userInfoSize is in bytes in the Java call (fitModel.userInfo.capacity()
        # elements of float); the buffer holds userInfoSize // 4 floats
        self.userInfo = np.zeros(max(0, userInfoSize) // 4 if userInfoSize >= 4 else 0, np.float32)


class FitResult:
    """GpufitImFCS.FitResult (GpufitImFCS.java:745-805)."""

    def __init__(self, numberFits, numberParameters):
        self.parameters = np.zeros(numberFits * numberParameters, np.float32)
        self.states = np.zeros(numberFits, np.int32)
        self.chiSquares = np.zeros(numberFits, np.float32)
        self.numberIterations = np.zeros(numberFits, np.int32)
        self.fitDuration = 0.0

    def isCompatible(self, numberFits, numberParameters):
        if self.parameters.size != numberFits * numberParameters:
            raise RuntimeError("Expected different size of parameters")
        if self.states.size != numberFits:
            raise RuntimeError("Expected different size of states")


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class GpufitImFCS:
    """Static entry points of gpufitImFCS.GpufitImFCS."""

    @staticmethod
    def fit(fitModel: FitModel, fitResult: FitResult | None = None) -> FitResult:
        if fitResult is None:
            fitResult = FitResult(fitModel.numberFits, fitModel.model.numberParameters)
        else:
            fitResult.isCompatible(fitModel.numberFits, fitModel.model.numberParameters)
        L = _lib.load()
        ui = np.ascontiguousarray(fitModel.userInfo, np.float32)
        t0 = time.time()
        status = L.imfcs_fit(fitModel.numberFits, fitModel.numberPoints, _p(fitModel.data),
                             _p(fitModel.weights), fitModel.model.id, _p(fitModel.initialParameters),
                             C.c_float(fitModel.tolerance), fitModel.maxNumberIterations,
                             fitModel.num_valid_coefs, _p(fitModel.parametersToFit), int(fitModel.estimator),
                             ui.nbytes, _p(ui), _p(fitResult.parameters), _p(fitResult.states),
                             _p(fitResult.chiSquares), _p(fitResult.numberIterations))
        fitResult.fitDuration = time.time() - t0
        if status != 0:
            raise RuntimeError(f"status = {status}, message = {GpufitImFCS.getLastError()}")
        return fitResult

    @staticmethod
    def getLastError() -> str:
        return _lib.last_error()

    @staticmethod
    def isCudaAvailable() -> bool:
        try:
            return bool(_lib.load().imfcs_is_cuda_available())
        except _lib.ImfcsError:
            return False

    @staticmethod
    def getCudaVersion() -> CudaVersion:
        rt, dr = C.c_int(0), C.c_int(0)
        if _lib.load().imfcs_get_cuda_version(C.byref(rt), C.byref(dr)) != 0:
            raise RuntimeError(GpufitImFCS.getLastError())

        def s(v):
            return f"{v // 1000}.{(v % 1000) // 10}"
        return CudaVersion(s(rt.value), s(dr.value))

    @staticmethod
    def resetGPU() -> None:
        _lib.load().imfcs_reset_gpu()

    @staticmethod
    def calcDataBleachCorrection(pixels: np.ndarray, outdata: np.ndarray, params: ACFParameters) -> None:
        src = _f32_in(pixels)
        GpufitImFCS._call("imfcs_calc_data_bleach_correction", _p(src), _f32_out(outdata), C.byref(params))

    @staticmethod
    def isBinningMemorySufficient(params: ACFParameters) -> bool:
        return bool(_lib.load().imfcs_is_binning_memory_sufficient(C.byref(params)))

    @staticmethod
    def calcBinning(indata: np.ndarray, outdata: np.ndarray, params: ACFParameters) -> None:
        src = _f32_in(indata)
        GpufitImFCS._call("imfcs_calc_binning", _p(src), _f32_out(outdata), C.byref(params))

    @staticmethod
    def isACFmemorySufficient(params: ACFParameters) -> bool:
        return bool(_lib.load().imfcs_is_acf_memory_sufficient(C.byref(params)))

    @staticmethod
    def calcACF(pixels, pixels1, blockvararray, NBmeanGPU, NBcovarianceGPU, blocked1D, bleachcorr_params,
                samp, lag, params: ACFParameters) -> None:
        def dptr(a):
            if a is None:
                return None
            assert a.dtype == np.float64 and a.flags.c_contiguous
            return C.c_void_p(a.ctypes.data)
        assert lag.dtype == np.int32
        src = _f32_in(pixels)
        GpufitImFCS._call("imfcs_calc_acf", _p(src), dptr(pixels1), dptr(blockvararray), dptr(NBmeanGPU),
                          dptr(NBcovarianceGPU), dptr(blocked1D), dptr(bleachcorr_params), dptr(samp),
                          C.c_void_p(lag.ctypes.data), C.byref(params))

    @staticmethod
    def _call(name, *args):
        if getattr(_lib.load(), name)(*args) != 0:
            raise RuntimeError(GpufitImFCS.getLastError())


def _f32_in(a) -> np.ndarray:
    """A contiguous float32 view or copy of an input array; the caller keeps
    it alive across the library call."""
    return np.ascontiguousarray(a, np.float32)


def _f32_out(a) -> C.c_void_p:
    """Output arrays are filled in place, so they must already be contiguous
    float32 (the Java float[] the native writes into)."""
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise ValueError("output arrays must be contiguous float32")
    return C.c_void_p(a.ctypes.data)
