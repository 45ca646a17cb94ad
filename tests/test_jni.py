"""The JNI shim (jni/imfcs_jni.c) driven through a mock JNIEnv.

CPU: the shim compiled against the project's jni.h stub and linked with a
recording fake of the library: field reads of GpufitImFCS.ACFParameters
(ints, doubles, the two booleans), pointer plumbing, copy-back release modes,
null buffers, exceptions with the library's message, fit()'s 0 / -1.
GPU: the same shim linked with libimfcs_gb300.so; calcACF and fit through
the mock JNIEnv give what the C ABI gives when called directly."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "jni", "imfcs_jni.c")
STUB = os.path.join(ROOT, "jni", "stub")
MOCK = os.path.join(ROOT, "tests", "jni", "mock_jni.c")
FAKE = os.path.join(ROOT, "tests", "jni", "fake_imfcs.c")
INC = os.path.join(ROOT, "include")

FIELDS = [("width", "I"), ("height", "I"), ("win_star", "I"), ("hin_star", "I"), ("w_temp", "I"),
          ("h_temp", "I"), ("pixbinX", "I"), ("pixbinY", "I"), ("binningX", "I"), ("binningY", "I"),
          ("firstframe", "I"), ("lastframe", "I"), ("framediff", "I"), ("cfXDistance", "I"),
          ("cfYDistance", "I"), ("correlatorp", "D"), ("correlatorq", "D"), ("frametime", "D"),
          ("background", "I"), ("mtab1", "D"), ("mtabchanumminus1", "D"), ("sampchanumminus1", "D"),
          ("chanum", "I"), ("isNBcalculation", "Z"), ("bleachcorr_gpu", "Z"), ("bleachcorr_order", "I"),
          ("nopit", "I"), ("ave", "I")]


def _compile(out, sources, extra=()):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    cmd = [cc, "-std=c11", "-O1", "-Wall", "-Werror", "-shared", "-fPIC", "-I", STUB, "-I", INC, *sources, "-o", out,
           *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _declare(L):
    vp = C.c_void_p
    L.mock_env.restype = vp
    for n in ("mock_float_array", "mock_double_array", "mock_int_array"):
        getattr(L, n).restype = vp
        getattr(L, n).argtypes = [vp, C.c_int]
    L.mock_direct.restype = vp
    L.mock_direct.argtypes = [vp]
    L.mock_object.restype = vp
    L.mock_set_field.argtypes = [vp, C.c_char_p, C.c_char, C.c_double]
    L.mock_string.restype = C.c_char_p
    L.mock_string.argtypes = [vp]
    L.mock_int_array_len.argtypes = [vp]
    L.mock_int_array_data.restype = C.POINTER(C.c_int)
    L.mock_int_array_data.argtypes = [vp]
    L.mock_exception.restype = C.c_char_p
    pre = "Java_gpufitImFCS_GpufitImFCS_"
    getattr(L, pre + "calcACF").argtypes = [vp] * 12
    getattr(L, pre + "calcBinning").argtypes = [vp] * 5
    getattr(L, pre + "calcDataBleachCorrection").argtypes = [vp] * 5
    getattr(L, pre + "isBinningMemorySufficient").argtypes = [vp] * 3
    getattr(L, pre + "isACFmemorySufficient").argtypes = [vp] * 3
    getattr(L, pre + "isBinningMemorySufficient").restype = C.c_uint8
    getattr(L, pre + "isACFmemorySufficient").restype = C.c_uint8
    getattr(L, pre + "isCudaAvailableInt").restype = C.c_uint8
    getattr(L, pre + "isCudaAvailableInt").argtypes = [vp, vp]
    getattr(L, pre + "getLastError").restype = vp
    getattr(L, pre + "getLastError").argtypes = [vp, vp]
    getattr(L, pre + "getCudaVersionAsArray").restype = vp
    getattr(L, pre + "getCudaVersionAsArray").argtypes = [vp, vp]
    getattr(L, pre + "resetGPU").argtypes = [vp, vp]
    getattr(L, pre + "fit").restype = C.c_int
    getattr(L, pre + "fit").argtypes = [vp, vp, C.c_int, C.c_int, vp, vp, C.c_int, vp, C.c_float, C.c_int, C.c_int, vp,
                               C.c_int, C.c_int, vp, vp, vp, vp, vp]
    return L


def _jobject_params(L, values: dict):
    o = L.mock_object()
    for name, sig in FIELDS:
        assert L.mock_set_field(o, name.encode(), sig.encode(), float(values.get(name, 0))) == 0
    return o


@pytest.fixture(scope="module")
def fake(tmp_path_factory):
    d = tmp_path_factory.mktemp("jni_fake")
    so = _compile(str(d / "libjni_fake.so"), [SHIM, MOCK, FAKE])
    L = _declare(C.CDLL(so))
    for n in ("fake_params",):
        getattr(L, n).argtypes = [C.POINTER(_lib.ACFParameters)]
    L.fake_ptr.restype = C.c_void_p
    L.fake_int.restype = C.c_long
    L.fake_tol.restype = C.c_float
    L.fake_last_call.restype = C.c_char_p
    return L


PRE = "Java_gpufitImFCS_GpufitImFCS_"


def _vals(**over):
    v = {name: i + 3 for i, (name, sig) in enumerate(FIELDS) if sig == "I"}
    v.update(correlatorp=16.0, correlatorq=8.0, frametime=1.25e-3, mtab1=2.0, mtabchanumminus1=128.0,
             sampchanumminus1=64.0, isNBcalculation=1, bleachcorr_gpu=0)
    v.update(over)
    return v


def test_shim_reads_every_parameter_field(fake):
    L = fake
    env = L.mock_env()
    L.mock_reset()
    vals = _vals(isNBcalculation=1, bleachcorr_gpu=1)
    prm = _jobject_params(L, vals)
    assert getattr(L, PRE + "isACFmemorySufficient")(env, None, prm) == 1
    got = _lib.ACFParameters()
    L.fake_params(C.byref(got))
    for name, sig in FIELDS:
        want = vals[name]
        if sig == "Z":
            want = 1 if want else 0
        assert getattr(got, name) == pytest.approx(want), name
    assert L.mock_bad_fields() == 0
    # booleans false -> 0
    prm = _jobject_params(L, _vals(isNBcalculation=0, bleachcorr_gpu=0))
    getattr(L, PRE + "isBinningMemorySufficient")(env, None, prm)
    L.fake_params(C.byref(got))
    assert got.isNBcalculation == 0 and got.bleachcorr_gpu == 0


def test_calc_acf_plumbing_and_copy_back(fake):
    L = fake
    env = L.mock_env()
    for bleach in (0, 1):
        L.mock_reset()
        L.fake_set_rc(0)
        px = np.arange(12, dtype=np.float32) + 5
        outs = [np.zeros(6) for _ in range(5)]
        bcp = np.array([9.0, 1.0])
        samp = np.zeros(4)
        lag = np.zeros(4, np.int32)
        objs = [L.mock_float_array(px.ctypes.data, px.size)] + \
               [L.mock_double_array(o.ctypes.data, o.size) for o in outs] + \
               [L.mock_double_array(bcp.ctypes.data, bcp.size), L.mock_double_array(samp.ctypes.data, samp.size),
                L.mock_int_array(lag.ctypes.data, lag.size)]
        prm = _jobject_params(L, _vals(bleachcorr_gpu=bleach))
        getattr(L, PRE + "calcACF")(env, None, *objs, prm)
        assert L.mock_exception() is None
        assert L.fake_last_call() == b"acf"
        assert L.fake_int(0) == 5                       # the pixels reached the library
        assert L.fake_int(1) == (9 if bleach else -1)   # coefficients only with bleachcorr_gpu
        assert [o[0] for o in outs] == [1.5, 2.5, 3.5, 4.5, 5.5]
        assert samp[0] == 6.5 and lag[0] == 7
        assert px[0] == 5 and bcp[0] == 9.0             # inputs untouched
        assert L.mock_release_count(0) == 7             # 5 doubles + samp + lag copied back
        assert L.mock_release_count(2) == 1 + bleach    # pixels (+ coefficients) aborted


def test_calc_acf_failure_throws_and_discards_outputs(fake):
    L = fake
    env = L.mock_env()
    L.mock_reset()
    L.fake_set_rc(1)
    px = np.ones(4, np.float32)
    acf = np.zeros(4)
    objs = [L.mock_float_array(px.ctypes.data, 4), L.mock_double_array(acf.ctypes.data, 4)] + [None] * 7
    getattr(L, PRE + "calcACF")(env, None, *objs, _jobject_params(L, _vals()))
    L.fake_set_rc(0)
    assert L.mock_exception() == b"java/lang/Exception: fake failure"
    assert acf[0] == 0.0                                # JNI_ABORT on failure
    assert L.fake_ptr(2) is None                        # null arrays pass as NULL


def test_binning_and_bleach_average(fake):
    L = fake
    env = L.mock_env()
    L.mock_reset()
    a = np.full(3, 4.0, np.float32)
    b = np.zeros(3, np.float32)
    getattr(L, PRE + "calcBinning")(env, None, L.mock_float_array(a.ctypes.data, 3), L.mock_float_array(b.ctypes.data, 3),
                           _jobject_params(L, _vals()))
    assert b[0] == 5.0 and a[0] == 4.0
    getattr(L, PRE + "calcDataBleachCorrection")(env, None, L.mock_float_array(a.ctypes.data, 3),
                                        L.mock_float_array(b.ctypes.data, 3), _jobject_params(L, _vals()))
    assert b[0] == 7.0
    assert L.mock_exception() is None


def test_fit_direct_buffers_and_status(fake):
    L = fake
    env = L.mock_env()
    bufs = [np.zeros(8, np.float32) for _ in range(9)]
    objs = [L.mock_direct(b.ctypes.data) for b in bufs]
    for rc, want in ((0, 0), (3, -1)):
        L.fake_set_rc(rc)
        got = getattr(L, PRE + "fit")(env, None, 11, 22, objs[0], None, 2, objs[2], C.c_float(1e-6), 33, 4, objs[3], 0, 88,
                             objs[4], objs[5], objs[6], objs[7], objs[8])
        assert got == want
    L.fake_set_rc(0)
    assert L.fake_ptr(0) == bufs[0].ctypes.data
    assert L.fake_ptr(1) is None                          # null weights buffer
    for i in (2, 3, 4, 5, 6, 7, 8):
        assert L.fake_ptr(i) == bufs[i].ctypes.data
    assert [L.fake_int(i) for i in range(7)] == [11, 22, 2, 33, 4, 0, 88]
    assert L.fake_tol() == pytest.approx(1e-6)


def test_status_natives(fake):
    L = fake
    env = L.mock_env()
    L.fake_set_rc(0)
    arr = getattr(L, PRE + "getCudaVersionAsArray")(env, None)
    assert L.mock_int_array_len(arr) == 2
    assert L.mock_int_array_data(arr)[0] == 13000
    assert getattr(L, PRE + "isCudaAvailableInt")(env, None) == 1
    L.fake_set_rc(1)
    assert getattr(L, PRE + "getCudaVersionAsArray")(env, None) is None
    assert L.mock_string(getattr(L, PRE + "getLastError")(env, None)) == b"fake failure"
    L.mock_reset()
    getattr(L, PRE + "resetGPU")(env, None)
    assert L.mock_exception() is not None
    L.fake_set_rc(0)


# ---------------------------------------------------------------------------
# GPU: the shim over the real library.
# ---------------------------------------------------------------------------


@pytest.fixture(scope="module")
def real(tmp_path_factory):
    lib = _lib.load()
    d = tmp_path_factory.mktemp("jni_real")
    libdir = os.path.dirname(_lib.LIB_PATH)
    so = _compile(str(d / "libagpufit.so"), [SHIM, MOCK],
                  ["-L", libdir, "-limfcs_gb300", f"-Wl,-rpath,{libdir}"])
    return _declare(C.CDLL(so)), lib


@pytest.mark.gpu
def test_calc_acf_through_jni_matches_c_abi(real):
    from tests.synth import brownian_stack
    L, lib = real
    env = L.mock_env()
    L.mock_reset()
    raw = brownian_stack(7, 6, 4000, seed=41, density=2.0, cps=3e4)
    pixels = np.ascontiguousarray(raw.astype(np.float32) - 100)
    vals = dict(width=7, height=6, win_star=7, hin_star=6, w_temp=7, h_temp=6, pixbinX=1, pixbinY=1,
                binningX=1, binningY=1, firstframe=1, lastframe=4000, framediff=4000, cfXDistance=0,
                cfYDistance=0, correlatorp=16, correlatorq=8, frametime=1e-3, background=100, chanum=73,
                isNBcalculation=0, bleachcorr_gpu=0, bleachcorr_order=0, nopit=1000, ave=4)
    outs_j = [np.zeros(73 * 42), np.zeros(73 * 42), np.zeros(42), np.zeros(42), np.zeros(2 * 42), np.zeros(73)]
    lag_j = np.zeros(73, np.int32)
    objs = [L.mock_float_array(pixels.ctypes.data, pixels.size)] + \
           [L.mock_double_array(o.ctypes.data, o.size) for o in outs_j[:5]] + \
           [None, L.mock_double_array(outs_j[5].ctypes.data, 73), L.mock_int_array(lag_j.ctypes.data, 73)]
    getattr(L, PRE + "calcACF")(env, None, *objs, _jobject_params(L, vals))
    assert L.mock_exception() is None, L.mock_exception()
    p = _lib.ACFParameters(**vals)
    outs_c = [np.zeros_like(o) for o in outs_j]
    lag_c = np.zeros(73, np.int32)
    rc = lib.imfcs_calc_acf(pixels.ctypes.data, *[o.ctypes.data for o in outs_c[:5]], None, outs_c[5].ctypes.data,
                            lag_c.ctypes.data, C.byref(p))
    assert rc == 0, _lib.last_error()
    for a, b in zip(outs_j, outs_c):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(lag_j, lag_c)
    assert np.isfinite(outs_j[0].reshape(73, 42)[1]).all()


@pytest.mark.gpu
def test_fit_through_jni_matches_c_abi(real):
    L, lib = real
    env = L.mock_env()
    rng = np.random.default_rng(3)
    nf, npts = 64, 40
    x = np.linspace(-1, 1, npts).astype(np.float32)
    coef = rng.normal(0, 1, (nf, 3))
    data = (coef[:, :1] + coef[:, 1:2] * x + coef[:, 2:3] * x ** 2 + rng.normal(0, 0.01, (nf, npts))).astype(np.float32)
    init = np.zeros((nf, 11), np.float32)
    to_fit = np.array([1, 1, 1] + [0] * 8, np.int32)

    def run(via_jni):
        outp = np.zeros((nf, 11), np.float32)
        st = np.zeros(nf, np.int32)
        chi = np.zeros(nf, np.float32)
        it = np.zeros(nf, np.int32)
        if via_jni:
            d = lambda a: L.mock_direct(a.ctypes.data)
            rc = getattr(L, PRE + "fit")(env, None, nf, npts, d(data), None, _lib.MODEL_LINEAR_1D, d(init), C.c_float(1e-6),
                                200, 3, d(to_fit), 0, npts * 4, d(x), d(outp), d(st), d(chi), d(it))
        else:
            rc = lib.imfcs_fit(nf, npts, data.ctypes.data, None, _lib.MODEL_LINEAR_1D, init.ctypes.data,
                               C.c_float(1e-6), 200, 3, to_fit.ctypes.data, 0, npts * 4, x.ctypes.data,
                               outp.ctypes.data, st.ctypes.data, chi.ctypes.data, it.ctypes.data)
        assert rc == 0, _lib.last_error()
        return outp, st, chi, it

    a, b = run(True), run(False)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    np.testing.assert_allclose(a[0][:, :3], coef, atol=0.05)
