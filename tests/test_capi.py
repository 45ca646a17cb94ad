"""CPU tests of the C ABI library: it builds, loads, exports every symbol the
public header declares, and its host-side validation rejects bad input with
the reference's messages -- without touching a GPU."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "imfcs_gb300.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"IMFCS_API\s+[\w\s\*]+?\b(imfcs_\w+)\s*\(", txt)))


def test_header_declares_the_documented_entry_points():
    syms = header_symbols()
    for s in ("imfcs_calc_acf", "imfcs_fit", "imfcs_calc_binning", "imfcs_calc_data_bleach_correction",
              "imfcs_is_acf_memory_sufficient", "imfcs_is_binning_memory_sufficient", "imfcs_get_last_error",
              "imfcs_is_cuda_available", "imfcs_get_cuda_version", "imfcs_reset_gpu", "imfcs_plan_create",
              "imfcs_plan_execute", "imfcs_plan_execute_host", "imfcs_diffusion_law", "imfcs_simulate"):
        assert s in syms


def test_library_exports_every_header_symbol():
    L = _lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (imfcs_\w+)", out))
    for s in header_symbols():
        assert s in exported, s
        assert hasattr(L, s)
    # nothing else leaks out of the library's C ABI namespace
    assert exported == set(header_symbols())


def test_binding_lists_every_export():
    assert sorted(_lib.EXPORTS) == header_symbols()


def test_struct_layouts_match_header():
    # the ctypes mirrors must have the field counts of the C structs
    txt = open(HEADER).read()
    assert C.sizeof(_lib.Outputs) == 13 * C.sizeof(C.c_void_p)
    assert "typedef struct imfcs_outputs" in txt
    assert len(_lib.ACFParameters._fields_) == 28


def test_chanum_matches_java_formula():
    L = _lib.load()
    for p, q in ((16, 8), (16, 7), (16, 2), (32, 8)):
        assert L.imfcs_chanum(p, q) == int(p + (q - 1) * p / 2 + 1)


def _plan_error(**kw):
    base = dict(width=8, height=8, frames=4000, background=100)
    base.update(kw)
    cfg = engine.FCSConfig(**base)
    with pytest.raises(_lib.ImfcsError) as e:
        engine.Plan(cfg)
    return str(e.value)


def test_rejects_too_few_frames():
    # java:7315 "Not enough frames": (T - 2^(Q-1) P/2 - P/4 2^Q) / 2^(Q-1) < 1
    assert "Not enough frames" in _plan_error(frames=2175, q=8)


def test_rejects_windows_outside_image():
    assert "outside the image" in _plan_error(binx=2, biny=2, out_w=5, out_h=4)
    assert "outside the image" in _plan_error(cfx=2, out_w=8)


def test_rejects_bad_polynomial_order():
    assert "polynomial order" in _plan_error(bleach=_lib.BLEACH_POLYNOMIAL, poly_order=9)


def test_rejects_bad_background_and_frame_range():
    assert "background" in _plan_error(background=-1)
    assert "frame range" in _plan_error(first=3990, num=100)


def test_without_gpu_compute_entry_points_fail_with_message():
    L = _lib.load()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    assert L.imfcs_is_cuda_available() == 0
    assert _lib.last_error() != ""
    cfg = engine.FCSConfig(width=8, height=8, frames=4000, background=100)
    with pytest.raises(_lib.ImfcsError):
        engine.Plan(cfg)   # device allocation fails: no CPU fallback
    rc = L.imfcs_fit(1, 4, None, None, 2, None, C.c_float(1e-4), 10, 0, None, 0, 0, None, None, None,
                     None, None)
    assert rc == -1 and "invalid argument" in _lib.last_error()


def test_model_constants_and_obsvol():
    import oracle
    cst = engine.model_constants(pixel_um=0.24, binx=2, biny=3, psf_um=0.4, cfx=1, cfy=0)
    assert cst[0] == pytest.approx(0.48e-6) and cst[1] == pytest.approx(0.72e-6)
    assert cst[4] == pytest.approx(0.24e-6) and cst[5] == 0
    assert cst[6] == pytest.approx(oracle.obsvol(cst[0], cst[1], cst[2]), rel=1e-14)


def test_config_defaults_follow_the_plugin():
    cfg = engine.FCSConfig(width=21, height=21, frames=20000)
    assert cfg.chanum == 73 and cfg.npix == 441
    assert cfg.init[0] == 1.0 and cfg.init[1] == 1e-12 and cfg.free_mask[:5] == (1, 1, 0, 0, 1)
    c = cfg.to_c()
    assert c.fitend == 72 and c.max_iter == 2000


@pytest.mark.gpu
def test_fp32_fma_probe_rate_is_plausible():
    """The FP32 issue-rate probe (the fit roofline's denominator) reports a
    rate between a few T and 100 T FMA/s on one GPU."""
    L = _lib.load()
    r = C.c_double()
    _lib.check(L.imfcs_measure_fp32_fma_rate(C.byref(r), None), "imfcs_measure_fp32_fma_rate")
    assert 5e12 < r.value < 1e14


def test_fp32_fma_probe_without_device():
    if torch_cuda_available():
        pytest.skip("a device is present")
    L = _lib.load()
    r = C.c_double()
    assert L.imfcs_measure_fp32_fma_rate(C.byref(r), None) != 0 and _lib.last_error()


def torch_cuda_available() -> bool:
    import torch
    return torch.cuda.is_available()
