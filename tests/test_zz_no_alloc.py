"""imfcs_fit_device_noalloc: the fit on device buffers with file-scope
scratch, for callers that cannot allocate device memory at fit time.
Compared with imfcs_fit (host buffers, allocating) on the same inputs, on two
calls in a row, at a small batch and at exactly the maximum batch; a warm call
must leave the device's free memory unchanged.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib
from tests.helpers import FIT_TOL
from tests.test_gpu_fit import _acf_curves


def test_noalloc_rejects_oversized_batch():
    L = _lib.load()
    n = 16385
    ptf = np.zeros(20, np.int32)
    dummy = C.c_void_p(1)      # never dereferenced: the size check comes first
    rc = L.imfcs_fit_device_noalloc(n, 72, dummy, None, 2, dummy, C.c_float(1e-6), 10, 0, ptf.ctypes.data,
                                    dummy, dummy, None, None, None, None)
    assert rc == -1
    assert "IMFCS_FIT_NOALLOC_MAX_FITS" in _lib.last_error()


@pytest.mark.gpu
def test_noalloc_fit_matches_allocating_fit():
    import torch
    L = _lib.load()
    n, npts = 64, 72
    data, var, lagtime, cst = _acf_curves(n, seed=5)
    y = np.ascontiguousarray(data[:, 1:], np.float32)
    w = np.ascontiguousarray(1.0 / var[:, 1:], np.float32)
    init = np.zeros((n, 20), np.float32)
    init[:, 0], init[:, 1] = 1.0, 1e-12
    init[:, 11:20] = cst
    ptf = np.zeros(20, np.int32)
    ptf[[0, 1, 4]] = 1
    x = np.ascontiguousarray(lagtime[1:], np.float32)

    # reference: the allocating host-buffer entry
    outp = np.zeros((n, 20), np.float32)
    st = np.zeros(n, np.int32)
    chi = np.zeros(n, np.float32)
    it = np.zeros(n, np.int32)
    rc = L.imfcs_fit(n, npts, y.ctypes.data, w.ctypes.data, 2, init.ctypes.data, C.c_float(1e-16), 2000, 0,
                     ptf.ctypes.data, 0, x.nbytes, x.ctypes.data, outp.ctypes.data, st.ctypes.data,
                     chi.ctypes.data, it.ctypes.data)
    assert rc == 0, _lib.last_error()

    dev = torch.device("cuda:0")
    d_y, d_w, d_init, d_x = (torch.from_numpy(a).to(dev) for a in (y, w, init, x))
    stream = torch.cuda.current_stream()
    for _ in range(2):                       # two calls in a row reuse the scratch
        d_out = torch.full((n, 20), float("nan"), device=dev)
        d_st = torch.full((n,), -7, dtype=torch.int32, device=dev)
        d_chi = torch.zeros(n, device=dev)
        d_it = torch.zeros(n, dtype=torch.int32, device=dev)
        rc = L.imfcs_fit_device_noalloc(n, npts, d_y.data_ptr(), d_w.data_ptr(), 2, d_init.data_ptr(),
                                        C.c_float(1e-16), 2000, 0, ptf.ctypes.data, d_x.data_ptr(),
                                        d_out.data_ptr(), d_st.data_ptr(), d_chi.data_ptr(), d_it.data_ptr(),
                                        C.c_void_p(stream.cuda_stream))
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        np.testing.assert_array_equal(d_st.cpu().numpy(), st)
        np.testing.assert_array_equal(got[:, 11:], init[:, 11:])
        np.testing.assert_allclose(got[:, [0, 1, 4]], outp[:, [0, 1, 4]], rtol=FIT_TOL, atol=1e-7)
        np.testing.assert_allclose(d_chi.cpu().numpy(), chi, rtol=1e-4)


@pytest.mark.gpu
def test_noalloc_linear_fit_matches_allocating_fit():
    import torch
    L = _lib.load()
    n, npts, ncoef = 16, 1000, 4
    rng = np.random.default_rng(9)
    x = np.ascontiguousarray(1e-3 * (np.arange(npts) + 0.5) * 20, np.float32)
    coefs = np.stack([rng.uniform(100, 500, n), rng.uniform(-5, -1, n), rng.uniform(0, .1, n),
                      rng.uniform(-1e-3, 0, n)], 1)
    y = np.stack([np.polynomial.polynomial.polyval(x.astype(float), c) for c in coefs]) + rng.normal(0, 1, (n, npts))
    y = np.ascontiguousarray(y, np.float32)
    init = np.zeros((n, 11), np.float32)
    init[:, 0] = y[:, -1]
    ptf = np.zeros(11, np.int32)
    ptf[:ncoef] = 1
    outp = np.zeros((n, 11), np.float32)
    rc = L.imfcs_fit(n, npts, y.ctypes.data, None, 3, init.ctypes.data, C.c_float(1e-6), 200, ncoef,
                     ptf.ctypes.data, 0, x.nbytes, x.ctypes.data, outp.ctypes.data, None, None, None)
    assert rc == 0, _lib.last_error()
    dev = torch.device("cuda:0")
    d_y, d_init, d_x = (torch.from_numpy(a).to(dev) for a in (y, init, x))
    for _ in range(2):
        d_out = torch.full((n, 11), float("nan"), device=dev)
        rc = L.imfcs_fit_device_noalloc(n, npts, d_y.data_ptr(), None, 3, d_init.data_ptr(), C.c_float(1e-6),
                                        200, ncoef, ptf.ctypes.data, d_x.data_ptr(), d_out.data_ptr(), None,
                                        None, None, None)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        for i in range(n):
            f_g = np.polynomial.polynomial.polyval(x.astype(float), got[i, :ncoef].astype(float))
            f_r = np.polynomial.polynomial.polyval(x.astype(float), outp[i, :ncoef].astype(float))
            assert np.max(np.abs(f_g - f_r)) <= 1e-5 * np.abs(f_r).max()


def _fit_inputs(n):
    base, var, lagtime, cst = _acf_curves(64, seed=5)
    reps = (n + 63) // 64
    data = np.tile(base, (reps, 1))[:n]
    var = np.tile(var, (reps, 1))[:n]
    y = np.ascontiguousarray(data[:, 1:], np.float32)
    w = np.ascontiguousarray(1.0 / var[:, 1:], np.float32)
    init = np.zeros((n, 20), np.float32)
    init[:, 0], init[:, 1] = 1.0, 1e-12
    init[:, 11:20] = cst
    x = np.ascontiguousarray(lagtime[1:], np.float32)
    return y, w, init, x


@pytest.mark.gpu
def test_noalloc_at_maximum_batch_allocates_nothing():
    import torch
    L = _lib.load()
    n, npts = 16384, 72                      # == IMFCS_FIT_NOALLOC_MAX_FITS
    y, w, init, x = _fit_inputs(n)
    ptf = np.zeros(20, np.int32)
    ptf[[0, 1, 4]] = 1
    outp = np.zeros((n, 20), np.float32)
    st = np.zeros(n, np.int32)
    rc = L.imfcs_fit(n, npts, y.ctypes.data, w.ctypes.data, 2, init.ctypes.data, C.c_float(1e-16), 2000, 0,
                     ptf.ctypes.data, 0, x.nbytes, x.ctypes.data, outp.ctypes.data, st.ctypes.data, None, None)
    assert rc == 0, _lib.last_error()
    dev = torch.device("cuda:0")
    d_y, d_w, d_init, d_x = (torch.from_numpy(a).to(dev) for a in (y, w, init, x))
    d_out = torch.full((n, 20), float("nan"), device=dev)
    d_st = torch.full((n,), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()

    def call():
        rc = L.imfcs_fit_device_noalloc(n, npts, d_y.data_ptr(), d_w.data_ptr(), 2, d_init.data_ptr(),
                                        C.c_float(1e-16), 2000, 0, ptf.ctypes.data, d_x.data_ptr(),
                                        d_out.data_ptr(), d_st.data_ptr(), None, None,
                                        C.c_void_p(stream.cuda_stream))
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()

    call()                                   # warm: module loading happens here
    free0 = torch.cuda.mem_get_info()[0]
    call()
    assert torch.cuda.mem_get_info()[0] == free0
    np.testing.assert_array_equal(d_st.cpu().numpy(), st)
    got = d_out.cpu().numpy()
    np.testing.assert_allclose(got[:, [0, 1, 4]], outp[:, [0, 1, 4]], rtol=FIT_TOL, atol=1e-7)
