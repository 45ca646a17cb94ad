"""Batches (imfcs_batch_*: binnings x cross-correlation offsets over one stack
as one CUDA graph) and the correlator tile autotuner (imfcs_plan_autotune).

A batch job runs the same kernels as a plan of the same config: its outputs
must equal the standalone plan's bit for bit, whatever the lane assignment,
and stay equal when the graph is re-captured for a new stack or new outputs.
Every correlator tile must meet the oracle parity bar."""
import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib, engine
from tests.helpers import ACF_TOL, VAR_TOL, acf_deviation, oracle_kwargs
from tests.synth import brownian_stack

W, H, T = 12, 10, 3000


def _jobs(**kw):
    return engine.batch_configs(W, H, T, binnings=(1, 2, 3), offsets=((0, 0), (1, 0), (1, 1)),
                                background=100, bleach=_lib.BLEACH_SINGLE_EXP, **kw)


def test_batch_configs_geometry():
    cfgs = engine.batch_configs(256, 256, 20000)
    assert len(cfgs) == 45
    first = cfgs[0]
    assert (first.out_w, first.out_h, first.npix) == (256, 256, 65536)
    c = next(c for c in cfgs if (c.binx, c.cfx, c.cfy) == (2, 2, 1))
    # the displaced window stays inside the frame
    assert (c.out_w - 1) * c.pixbinx + c.cfx + c.binx <= 256
    assert (c.out_h - 1) * c.pixbiny + c.cfy + c.biny <= 256
    assert c.cst[4] == pytest.approx(0.24e-6 * 2) and c.cst[5] == pytest.approx(0.24e-6)


def test_batch_rejects_jobs_on_different_stacks():
    a = engine.FCSConfig(width=W, height=H, frames=T)
    b = engine.FCSConfig(width=W, height=H, frames=T - 100)
    with pytest.raises(_lib.ImfcsError, match="same stack"):
        engine.Batch([a, b])


def _plan_outputs(cfg, dev_stack, tile=None):
    import torch
    plan = engine.Plan(cfg)
    try:
        if tile is not None:
            plan.set_corr_tile(*tile)
        out = plan.alloc_device_outputs()
        plan.execute(dev_stack, out)
        plan.synchronize()
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in out.items()}
    finally:
        plan.close()


def _dev(stack):
    import torch
    return torch.from_numpy(stack.view(np.int16)).cuda().view(torch.uint16)


def _assert_same(a, b):
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [1, 3])
def test_batch_equals_standalone_plans(lanes):
    import torch
    stack = brownian_stack(W, H, T, seed=21, density=2.0, cps=3e4, tau_bleach=15.0)
    cfgs = _jobs()
    dev = _dev(stack)
    ref = [_plan_outputs(c, dev) for c in cfgs]
    batch = engine.Batch(cfgs, lanes=lanes)
    try:
        assert batch.lanes == lanes
        outs = batch.alloc_device_outputs()
        for _ in range(2):                       # capture, then replay
            for o in outs:
                for v in o.values():
                    v.fill_(0)
            batch.execute(dev, outs)
            batch.synchronize()
            torch.cuda.synchronize()
            for r, o in zip(ref, outs):
                _assert_same(r, {k: v.cpu().numpy() for k, v in o.items()})
        assert batch.kernel_launches() > 10 * len(cfgs)
        # a new stack and new outputs: the graph is captured again
        stack2 = brownian_stack(W, H, T, seed=22, density=2.0, cps=3e4, tau_bleach=15.0)
        dev2 = _dev(stack2)
        ref2 = [_plan_outputs(c, dev2) for c in cfgs]
        outs2 = batch.alloc_device_outputs()
        batch.execute(dev2, outs2)
        batch.synchronize()
        torch.cuda.synchronize()
        for r, o in zip(ref2, outs2):
            _assert_same(r, {k: v.cpu().numpy() for k, v in o.items()})
    finally:
        batch.close()


@pytest.mark.gpu
def test_batch_gls_jobs_equal_standalone_plans():
    import torch
    stack = brownian_stack(W, H, T, seed=23, density=2.0, cps=3e4)
    cfgs = engine.batch_configs(W, H, T, binnings=(1, 2), offsets=((0, 0), (1, 0)), background=100, gls=True)
    dev = _dev(stack)
    ref = [_plan_outputs(c, dev) for c in cfgs]
    batch = engine.Batch(cfgs, lanes=2)
    try:
        outs = batch.alloc_device_outputs()
        batch.execute(dev, outs)
        batch.synchronize()
        torch.cuda.synchronize()
        for r, o in zip(ref, outs):
            _assert_same(r, {k: v.cpu().numpy() for k, v in o.items()})
    finally:
        batch.close()


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [(64, 0, 0), (64, 1, 1), (64, 2, 2), (32, 0, 0), (32, 1, 1), (32, 2, 2),
                                  (64, 0, 3), (64, 1, 4), (32, 2, 0)])
@pytest.mark.parametrize("kw", [{}, {"cfx": 1, "cfy": 1}, {"binx": 2, "biny": 2}], ids=["acf", "ccf11", "bin2"])
def test_corr_tiles_match_oracle(tile, kw):
    import oracle
    stack = brownian_stack(W, H, T, seed=24, density=2.0, cps=3e4, tau_bleach=15.0)
    # polynomial bleach: a least-squares solve, so the corrected traces do not
    # depend on where an optimiser stops (the tile changes only the correlator)
    cfg = engine.FCSConfig(width=W, height=H, frames=T, background=100, bleach=_lib.BLEACH_POLYNOMIAL,
                           do_fit=False, **kw)
    gpu = _plan_outputs(cfg, _dev(stack), tile)
    ref = oracle.run(stack, **oracle_kwargs(cfg))
    np.testing.assert_array_equal(gpu["blocked_ind"], ref["blocked_ind"])
    np.testing.assert_array_equal(np.isfinite(gpu["acf"]), np.isfinite(ref["acf"]))
    assert acf_deviation(gpu, ref) <= ACF_TOL
    v_g, v_r = gpu["var"][:, 1:], ref["var"][:, 1:]
    fin = np.isfinite(v_r)
    rel = np.abs(v_g[fin] - v_r[fin]) / np.abs(v_r[fin])
    assert rel.max() <= VAR_TOL


@pytest.mark.gpu
def test_plan_autotune_keeps_a_measured_tile():
    import torch
    stack = brownian_stack(W, H, T, seed=25, density=2.0, cps=3e4)
    cfg = engine.FCSConfig(width=W, height=H, frames=T, background=100)
    dev = _dev(stack)
    plan = engine.Plan(cfg)
    try:
        out = plan.alloc_device_outputs()
        trials = plan.autotune(dev, out)
        assert len(trials) == 10 and all(t["ms"] > 0 for t in trials)
        best = min(trials, key=lambda t: t["ms"])
        assert plan.corr_tile() == (best["cta"], best["seg_extra"], best["tail_extra"])
        plan.execute(dev, out)
        plan.synchronize()
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in out.items()}
    finally:
        plan.close()
    _assert_same(_plan_outputs(cfg, dev, (best["cta"], best["seg_extra"], best["tail_extra"])), got)


@pytest.mark.gpu
def test_batch_autotune_lanes_and_results():
    import torch
    stack = brownian_stack(W, H, T, seed=26, density=2.0, cps=3e4, tau_bleach=15.0)
    cfgs = _jobs()
    dev = _dev(stack)
    batch = engine.Batch(cfgs, lanes=1)
    try:
        outs = batch.alloc_device_outputs()
        lane_ms = batch.autotune(dev, outs, max_lanes=3)
        assert all(t > 0 for t in lane_ms)
        assert batch.lanes == 1 + int(np.argmin(lane_ms))
        infos = [batch.job_info(i) for i in range(len(cfgs))]
        assert all(i["ms"] > 0 for i in infos)
        batch.execute(dev, outs)
        batch.synchronize()
        torch.cuda.synchronize()
        for c, i, o in zip(cfgs, infos, outs):
            _assert_same(_plan_outputs(c, dev, (i["cta"], i["seg_extra"], i["tail_extra"])),
                         {k: v.cpu().numpy() for k, v in o.items()})
    finally:
        batch.close()
