"""Stack ingest (imfcs_tiff_*) and background-file statistics
(imfcs_background_stats, loadBGRFile java:6988-7103).

The TIFF files are written here by a small independent writer: one IFD per
frame with several strips, in both byte orders, and ImageJ's single-IFD
stack layout ("images=N", frames contiguous).  Reading is host code, so it
is tested without a GPU; the device path and the statistics run on the GPU
and must equal the Java-order FP64 restatement bit for bit."""
import struct

import numpy as np
import pytest

import oracle
from imaging_fcs_1_52_gb300 import _lib
from imaging_fcs_1_52_gb300.ingest import TiffStack, background_stats


def write_tiff(path, stack, order="<", layout="pages", strips=3, bits=16, compression=1, description=None):
    """Baseline TIFF writer: `layout` "pages" (one IFD per frame, the frame
    split into `strips` strips) or "imagej" (one IFD, ImageJ description,
    all frames contiguous after the IFD)."""
    f, h, w = stack.shape
    bom = b"II" if order == "<" else b"MM"
    dt = np.dtype(order + "u2")
    out = bytearray(bom + struct.pack(order + "HI", 42, 0))

    def entry(tag, typ, count, value):
        if typ == 3 and count == 1:
            return struct.pack(order + "HHIH2x", tag, typ, count, value)
        return struct.pack(order + "HHII", tag, typ, count, value)

    def put_ifd(entries, next_off_pos_holder):
        pos = len(out)
        out.extend(struct.pack(order + "H", len(entries)))
        for e in entries:
            out.extend(e)
        next_pos = len(out)
        out.extend(struct.pack(order + "I", 0))
        return pos, next_pos

    prev_next = 4
    frames = range(f) if layout == "pages" else range(1)
    desc = description
    if layout == "imagej" and desc is None:
        desc = f"ImageJ=1.54f\nimages={f}\nslices={f}\nloop=false\n"
    for z in frames:
        data = stack[z].astype(dt).tobytes() if layout == "pages" else stack.astype(dt).tobytes()
        rows = np.array_split(np.arange(h), strips if layout == "pages" else 1)
        offs, cnts = [], []
        for r in rows:
            offs.append(len(out))
            seg = data[r[0] * w * 2:(r[-1] + 1) * w * 2]
            if layout == "imagej":
                seg = data
            out.extend(seg)
            cnts.append(len(seg) if layout == "pages" else h * w * 2)
        if len(out) % 2:
            out.append(0)
        arr_off = len(out)
        for o in offs:
            out.extend(struct.pack(order + "I", o))
        cnt_off = len(out)
        for c in cnts:
            out.extend(struct.pack(order + "I", c))
        desc_off = len(out)
        if desc is not None and z == 0:
            out.extend(desc.encode() + b"\0")
        if len(out) % 2:
            out.append(0)
        n = len(offs)
        ents = [entry(256, 3, 1, w), entry(257, 3, 1, h), entry(258, 3, 1, bits), entry(259, 3, 1, compression),
                entry(262, 3, 1, 1)]
        if desc is not None and z == 0:
            ents.append(entry(270, 2, len(desc) + 1, desc_off))
        ents += [entry(273, 4, n, offs[0] if n == 1 else arr_off), entry(277, 3, 1, 1),
                 entry(278, 3, 1, h if n == 1 else len(rows[0])),
                 entry(279, 4, n, cnts[0] if n == 1 else cnt_off)]
        pos, next_pos = put_ifd(ents, None)
        struct.pack_into(order + "I", out, prev_next, pos)
        prev_next = next_pos
    with open(path, "wb") as fh:
        fh.write(out)


def _stack(f=7, h=5, w=6, seed=0):
    return np.random.default_rng(seed).integers(0, 65536, (f, h, w), dtype=np.uint16)


@pytest.mark.parametrize("order", ["<", ">"], ids=["le", "be"])
@pytest.mark.parametrize("layout,strips", [("pages", 1), ("pages", 3), ("imagej", 1)])
def test_tiff_read_roundtrip(tmp_path, order, layout, strips):
    st = _stack()
    p = tmp_path / "s.tif"
    write_tiff(p, st, order=order, layout=layout, strips=strips)
    with TiffStack(p) as t:
        assert (t.frames, t.height, t.width) == st.shape
        np.testing.assert_array_equal(t.read(), st)
        np.testing.assert_array_equal(t.read(2, 3), st[2:5])
        np.testing.assert_array_equal(t.read(6, 1), st[6:7])
        with pytest.raises(_lib.ImfcsError, match="frame range"):
            t.read(5, 3)


@pytest.mark.parametrize("kw,msg", [
    ({"bits": 8}, "16-bit"),
    ({"compression": 5}, "compressed"),
], ids=["8bit", "lzw"])
def test_tiff_rejects_unsupported(tmp_path, kw, msg):
    p = tmp_path / "bad.tif"
    write_tiff(p, _stack(), **kw)
    with pytest.raises(_lib.ImfcsError, match=msg):
        TiffStack(p)


def test_tiff_rejects_truncated_and_foreign(tmp_path):
    st = _stack(f=4)
    p = tmp_path / "t.tif"
    write_tiff(p, st, layout="imagej")
    data = p.read_bytes()
    (tmp_path / "short.tif").write_bytes(data[:len(data) - 10])
    with pytest.raises(_lib.ImfcsError, match="truncated|shorter"):
        TiffStack(tmp_path / "short.tif")
    # an ImageJ description claiming more frames than the file holds
    write_tiff(tmp_path / "claims.tif", st, layout="imagej", description="ImageJ=1.54f\nimages=10\n")
    with pytest.raises(_lib.ImfcsError, match="shorter"):
        TiffStack(tmp_path / "claims.tif")
    (tmp_path / "x.tif").write_bytes(b"GIF89a" + bytes(20))
    with pytest.raises(_lib.ImfcsError, match="not a TIFF"):
        TiffStack(tmp_path / "x.tif")
    with pytest.raises(_lib.ImfcsError, match="cannot open"):
        TiffStack(tmp_path / "missing.tif")


def test_oracle_background_stats_definitions():
    st = _stack(f=50, h=3, w=4, seed=3) // 100
    r = oracle.background_stats(st)
    x = st.astype(float)
    np.testing.assert_allclose(r["mean"], x.mean(0), rtol=1e-14)
    np.testing.assert_allclose(r["var"], x.var(0), rtol=1e-9)
    cov = (x[:-1] * x[1:]).mean(0) - x[:-1].mean(0) * x[1:].mean(0)
    np.testing.assert_allclose(r["covar"], cov, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(r["row_mean"], x.mean(axis=(0, 2)), rtol=1e-13)
    np.testing.assert_allclose(r["col_mean"], x.mean(axis=(0, 1)), rtol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["pages", "imagej"])
def test_tiff_read_device(tmp_path, layout):
    import torch
    st = _stack(f=300, h=33, w=40, seed=5)
    p = tmp_path / "d.tif"
    write_tiff(p, st, order=">", layout=layout)
    with TiffStack(p) as t:
        dev = t.read_device(10, 250)
        torch.cuda.synchronize()
        got = dev.view(torch.int16).cpu().numpy().view(np.uint16)
    np.testing.assert_array_equal(got, st[10:260])


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(2, 1, 1), (40, 7, 9), (1000, 16, 24)])
def test_background_stats_match_java_order(shape):
    import torch
    st = _stack(*shape, seed=7)
    dev = torch.from_numpy(st.view(np.int16)).cuda().view(torch.uint16)
    got = background_stats(dev)
    ref = oracle.background_stats(st)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.gpu
def test_background_file_feeds_the_plan(tmp_path):
    """The mean image of a background stack read from TIFF, as the plan's
    per-pixel background (the plugin's Bgr FILE mode)."""
    from imaging_fcs_1_52_gb300 import engine
    from tests.helpers import ACF_TOL, acf_deviation, oracle_kwargs
    from tests.synth import brownian_stack
    rng = np.random.default_rng(9)
    bg_stack = (100 + rng.integers(-2, 3, (200, 8, 10))).astype(np.uint16)
    p = tmp_path / "bg.tif"
    write_tiff(p, bg_stack, layout="imagej")
    with TiffStack(p) as t:
        bg = background_stats(t.read_device())
    st = brownian_stack(10, 8, 6000, seed=13, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(width=10, height=8, frames=6000, background=100)
    plan = engine.Plan(cfg)
    try:
        plan.set_background_image(bg["mean"])
        gpu = plan.execute_host(st)
    finally:
        plan.close()
    ref = oracle.run(st, **oracle_kwargs(cfg), bgr=np.floor(bg["mean"] + 0.5).astype(np.int32))
    assert acf_deviation(gpu, ref) <= ACF_TOL
