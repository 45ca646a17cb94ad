"""Benchmark: ACF + fit pixels/s on a 128 x 128 x 50,000-frame uint16 stack.

Workload (the plain method at scale): a seeded 2D Brownian simulation
(tests/synth_host.c, D drawn per 16 x 16 tile from U(0.2, 5) um^2/s,
single-exponential bleach tau = 20 s, 500 particles per 30 x 30 um, PSF
1/e^2 radius 0.4 um, 10,000 photons/s per particle, offset 100), all-pixel
multi-tau ACFs (P=16, Q=8, 73 channels) with blocked variance,
single-exponential bleach correction, and a batched LM fit of the TIRF
one-component model (N, D, G free) of every pixel.  Both arms read the same
stack (same generator, same seed).

One step = the whole path over the full stack.  `value` is measured with the
stack resident in HBM (1.64 GB, larger than L2, so no flush is needed);
`e2e` goes through the C ABI with host buffers every step
(imfcs_plan_execute_host_async: pinned host stack -> device on the plan's
copy stream, run, results -> pinned host buffers; the next step's stack copy
overlaps this step's run), synchronised once after the timed steps.

--impl reference runs the reference's CPU implementation of the path: the
Java CPU code cannot run here (no JVM), so the FP64 C restatement in oracle/
stands in for it, with all host threads (OpenMP), on a bounded sample (a band
of rows) of the same stack.

The GPU arm also compares its outputs on the CPU-baseline sample with the
oracle's (the `parity` block): blocking index and flag, fitted mask, ACF,
blocked variance, fitted N and D.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = H = 128
T = 50000
METRIC = "ACF+fit pixels/s at 128²×50k frames"
UNIT = "pixels/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=0, help="pixels in the CPU baseline sample (0: auto)")
    ap.add_argument("--frames", type=int, default=50000,
                    help="frames of the stack (50000 is the benchmark; fewer only for profiling captures)")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the multi-job block (256x256x20000, binnings 1-5 x offsets {0,1,2}^2, GLS)")
    a = ap.parse_args()
    global T
    T = a.frames
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_config(engine, lib):
    return engine.FCSConfig(width=W, height=H, frames=T, background=100, bleach=lib.BLEACH_SINGLE_EXP,
                            p=16, q=8, frametime=1e-3, do_fit=True,
                            cst=engine.model_constants(pixel_um=0.24, psf_um=0.4))


def host_stack(seed):
    from tests.synth import bench_stack
    return bench_stack(W, H, T, seed=seed)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and "Active" in r[3 + i]
                          and "Not" not in r[3 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_profile_traffic():
    """DRAM bytes per correlator-path launch (scaled to the full workload)
    from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "correlator_path_traffic.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["bytes_per_launch_full_size"])
        except Exception:
            return None
    return None


def cpu_baseline(stack_np, cfg, sample_pixels, threads):
    """The FP64 oracle (restatement of the Java CPU path) on a bounded sample
    of the same workload: the first sample_pixels pixels (whole rows), all
    frames.  Returns (pixels/s, pixels, seconds, oracle outputs)."""
    import oracle  # checker / baseline only
    ncols = min(sample_pixels, W)
    nrows = max(1, sample_pixels // ncols)
    sub = np.ascontiguousarray(stack_np[:, :nrows, :ncols])
    t0 = time.perf_counter()
    ref = oracle.run(sub, out_w=ncols, out_h=nrows, background=cfg.background, p=cfg.p, q=cfg.q,
                     frametime=cfg.frametime, bleach=cfg.bleach, init=np.array(cfg.init),
                     free_mask=np.array(cfg.free_mask, np.int32), cst=cfg.cst, threads=threads)
    dt = time.perf_counter() - t0
    return ncols * nrows / dt, ncols * nrows, dt, ref


def parity_block(gpu, ref, n, sel=None):
    """GPU outputs of the first n pixels against the oracle's on the same
    pixels (restricted to the pixels `sel` when given)."""
    g = {k: v[:n] for k, v in gpu.items()}
    if sel is not None:
        g = {k: v[sel] for k, v in g.items()}
        ref = {k: v[sel] for k, v in ref.items() if hasattr(v, "shape") and len(v) == n}
        n = int(sel.sum())
    out = {"pixels": int(n)}
    out["blocked_ind_equal"] = int((g["blocked_ind"] == ref["blocked_ind"]).sum())
    out["blocked_ok_equal"] = int((g["blocked_ok"] == ref["blocked_ok"]).sum())
    out["fitted_gpu"] = int(g["fitted"].sum())
    out["fitted_oracle"] = int(ref["fitted"].sum())
    out["fitted_equal"] = int((g["fitted"] == ref["fitted"]).sum())
    fin_r = np.all(np.isfinite(ref["acf"][:, 1:]), axis=1)
    fin_g = np.all(np.isfinite(g["acf"][:, 1:]), axis=1)
    out["acf_all_lags_finite_oracle"] = int(fin_r.sum())
    out["acf_finiteness_equal"] = int((np.isfinite(ref["acf"]) == np.isfinite(g["acf"])).all(axis=1).sum())
    both = fin_r & fin_g
    if both.any():
        dev = np.abs(g["acf"][both, 1:] - ref["acf"][both, 1:]) / np.abs(ref["acf"][both, 1:2])
        out["acf_max_dev_rel_g1"] = float(dev.max())
        vr, vg = ref["var"][both, 1:], g["var"][both, 1:]
        rel = np.abs(vg - vr) / np.abs(vr)
        out["var_max_rel"] = float(rel.max())
        out["var_median_rel"] = float(np.median(rel))
    fb = (g["fitted"] == 1) & (ref["fitted"] == 1)
    out["fitted_both"] = int(fb.sum())
    if fb.any():
        for i, name in ((0, "N"), (1, "D")):
            e = np.abs(g["fitres"][fb, i] - ref["fitres"][fb, i]) / np.abs(ref["fitres"][fb, i])
            out[f"{name}_max_rel"] = float(e.max())
            out[f"{name}_over_1e-4"] = int((e > 1e-4).sum())
        c = np.abs(g["chi2"][fb] - ref["chi2"][fb]) / np.abs(ref["chi2"][fb])
        out["chi2_max_rel"] = float(c.max())
    out["not_fitted_with_nonfinite_acf_oracle"] = int(((ref["fitted"] == 0) & ~fin_r).sum())
    return out


def reference_arm(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    from imaging_fcs_1_52_gb300 import engine, _lib  # configuration only
    cfg = make_config(engine, _lib)
    sample = args.cpu_sample or 1024
    stack_np = host_stack(seed=1)           # the GPU arm's stack (same generator, same seed)
    vals = []
    for i in range(args.warmup + args.steps):
        v, n, dt, _ = cpu_baseline(stack_np, cfg, sample, threads)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sample / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (tests/synth_host.c, seed 1: the GPU arm's stack)",
            "config": {"workload": f"128x128x{T} uint16 stack; single-exp bleach; P=16 Q=8 (73 ch); "
                                   "blocked variance; OLS LM TIRF fit (N, D, G)",
                       "sample": f"first {sample} pixels (rows 0..{sample // W - 1}) x {T} frames of that stack"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{sample} pixels x {T} frames, FP64 C restatement of the Java CPU path"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def surrogate_block(plan, stack, steps):
    """Surrogate-seeded LM against plain LM on the same correlator outputs:
    fit-stage device time (features + MLP + seeded LM + refits in the seeded
    mode), fitted pixels/s, and agreement at equal chi^2 (mode 1: refit of
    failed seeded fits; mode 2: plain LM also runs and arbitrates every pixel)."""
    import torch
    from imaging_fcs_1_52_gb300 import surrogate
    if not os.path.exists(surrogate.DEFAULT_WEIGHTS):
        return {"unavailable": "no trained weights (python -m imaging_fcs_1_52_gb300.train_surrogate)"}
    sur = surrogate.Surrogate.load()

    def run(mode):
        plan.set_surrogate(sur if mode else None, mode)
        o = plan.alloc_device_outputs()
        plan.execute(stack, o)
        ts = []
        for _ in range(max(3, steps)):
            plan.execute(stack, o)
            torch.cuda.synchronize()
            ts.append(plan.stage_times()["fits"])
        st = plan.surrogate_stats() if mode else {}
        return {k: v.cpu().numpy() for k, v in o.items()}, statistics.median(ts), st

    p_np, p_ms, _ = run(0)
    blk = {"weights": os.path.relpath(surrogate.DEFAULT_WEIGHTS, os.path.dirname(os.path.abspath(__file__))),
           "training": sur.meta.get("data", {}).get("curves"),
           "plain": {"fits_ms": p_ms, "fitted": int(p_np["fitted"].sum()),
                     "fitted_pixels_per_s": float(p_np["fitted"].sum()) / (p_ms * 1e-3),
                     "iterations_mean": float(p_np["iterations"].mean())}}
    for mode in (1, 2):
        s_np, s_ms, st = run(mode)
        both = (p_np["fitted"] == 1) & (s_np["fitted"] == 1)
        cr = s_np["chi2"][both] / p_np["chi2"][both]
        d = {"fits_ms": s_ms, "fitted": int(s_np["fitted"].sum()),
             "fitted_pixels_per_s": float(s_np["fitted"].sum()) / (s_ms * 1e-3),
             "speedup_vs_plain": p_ms / s_ms, "iterations_mean": float(s_np["iterations"].mean()),
             "refit": st.get("refit"), "worse_than_plain_refit": st.get("worse_than_plain"),
             "fitted_equal": int((s_np["fitted"] == p_np["fitted"]).sum()), "fitted_both": int(both.sum()),
             "chi2_within_1pct": int((cr <= 1.01).sum()), "chi2_ratio_max": float(cr.max()) if both.any() else None,
             "chi2_ratio_min": float(cr.min()) if both.any() else None}
        for i, nm in ((0, "N"), (1, "D")):
            rel = np.abs(s_np["fitres"][both, i] / p_np["fitres"][both, i] - 1)
            d[f"{nm}_rel_p99"] = float(np.quantile(rel, 0.99)) if both.any() else None
            d[f"{nm}_over_1e-4"] = int((rel > 1e-4).sum())
        blk[f"seeded_mode{mode}"] = d
    plan.set_surrogate(None)
    return blk


# FP32 operations of one point in one LM iteration of lm_tirf_kernel (the
# default one-component model, counted in its source, transcendentals as
# one): the model value and Jacobian -- tirf_terms 37 (p0 and 1/p0 5, the
# square-pixel lateral factor 11, its derivative chain 7, axial factor and
# derivative 9, products 5), tirf_f 7 -- plus the normal equations of K = 3
# free parameters, 2K + K(K+1) = 18.
FIT_OPS_PER_POINT_ITERATION = 37 + 7 + 18
MLP_FLOP_PER_SAMPLE = 2 * (128 * 256 + 256 * 256 + 256 * 4)   # forward GEMMs


def compute_rooflines(L, cfg, fits_ms, iterations_total):
    """Fit stage against the FP32 issue rate (measured by the library's FMA
    probe; one FMA = one operation) and the surrogate's forward pass against
    the measured bf16 tensor peak."""
    import ctypes as C
    import torch
    from imaging_fcs_1_52_gb300 import _lib, surrogate
    out = {}
    rate = C.c_double()
    _lib.check(L.imfcs_measure_fp32_fma_rate(C.byref(rate), None), "imfcs_measure_fp32_fma_rate")
    peak_g = rate.value / 1e9
    npts = (cfg.chanum - 1 if cfg.fitend is None else cfg.fitend) - cfg.fitstart + 1
    ops = float(iterations_total) * npts * FIT_OPS_PER_POINT_ITERATION
    ach = ops / (fits_ms * 1e-3) / 1e9
    out["fit"] = {"kernel": "fit stage (ols_prepare, lm_tirf_kernel, fit_epilogue)", "bound": "fp32 issue",
                  "unit": "G FP32 op/s", "achieved": ach, "peak": peak_g, "frac": ach / peak_g,
                  "peak_kind": "measured (FMA probe)", "ops_per_point_iteration": FIT_OPS_PER_POINT_ITERATION,
                  "points": npts, "iterations_total": int(iterations_total), "fits_ms": fits_ms}
    if os.path.exists(surrogate.DEFAULT_WEIGHTS):
        sur = surrogate.Surrogate.load()
        n = cfg.npix
        x = torch.randn((n, 128), device="cuda")
        sur.predict(x)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ts = []
        for _ in range(10):
            e0.record()
            sur.predict(x)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = statistics.median(ts)
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] \
            if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
        tf = MLP_FLOP_PER_SAMPLE * n / (ms * 1e-3) / 1e12
        out["mlp"] = {"kernel": "surrogate predict (standardise, 3 bf16 mma.sync GEMMs with fused epilogues)",
                      "bound": "tensor", "unit": "TFLOP/s", "achieved": tf, "peak": peak, "frac": tf / peak,
                      "rows": n, "ms": ms, "flop_per_row": MLP_FLOP_PER_SAMPLE}
    return out


def bands_block(engine, cfg, host_np, whole_out, tile, steps):
    """Band-streamed host execution (imfcs_bands_*) of the same pinned stack
    under a device budget of a quarter of the one-band footprint, with the
    whole-stack plan's correlator tile: bands, host-to-device time included,
    and its results against the whole-stack host execution's."""
    import torch
    try:
        one = engine.Bands(cfg, band_rows=cfg.out_h)
        full = one.geometry()["device_bytes"]
        one.close()
        bands = engine.Bands(cfg, max_device_bytes=full // 4)
        bands.set_corr_tile(*tile)
        tdt = {"f8": torch.float64, "f4": torch.float32, "i4": torch.int32}
        outs = {n: torch.empty(v.shape, dtype=tdt[v.dtype.str[1:]], pin_memory=True).numpy()
                for n, v in whole_out.items()}
        bands.execute_host(host_np, outs)            # warm-up
        t0 = time.perf_counter()
        for _ in range(steps):
            bands.execute_host(host_np, outs)
        ms = (time.perf_counter() - t0) * 1e3 / steps
        equal = all(np.array_equal(outs[n], whole_out[n], equal_nan=outs[n].dtype.kind == "f") for n in outs)
        fin = np.isfinite(whole_out["acf"]) & np.isfinite(outs["acf"])
        dev = float(np.abs(outs["acf"][fin] - whole_out["acf"][fin]).max()) if fin.any() else 0.0
        g = bands.geometry()
        bands.close()
        return {"budget_bytes": full // 4, "one_band_bytes": full, **g, "ms_per_step": ms,
                "pixels_per_s": cfg.npix / (ms * 1e-3), "equal_to_whole_stack": bool(equal),
                "acf_max_abs_dev": dev}
    except Exception as e:   # reported, never fatal to the bench line
        return {"error": str(e)}


def batch_block(steps):
    """Multi-job batch: a 256x256x20000 two-component stack (D1 = 0.5,
    D2 = 5 um^2/s, 70/30, GPU Monte-Carlo simulator), binnings 1-5 x
    cross-correlation offsets (dx, dy) in {0,1,2}^2 = 45 jobs, each with the
    GLS covariance (72x72 FP64 Cholesky + shrinkage) and the GLS fit, run as
    one CUDA graph.  Autotuned correlator tiles and lane count; the graph's
    time is set against the sum of the jobs' own times (each job executed
    alone with eager launches)."""
    import torch
    from imaging_fcs_1_52_gb300 import engine
    Wb, Hb, Tb = 256, 256, 20000
    t0 = time.perf_counter()
    stack = engine.simulate(Wb, Hb, Tb, d1=0.5, d2=5.0, fraction2=0.3, seed=3)
    torch.cuda.synchronize()
    sim_s = time.perf_counter() - t0
    cfgs = engine.batch_configs(Wb, Hb, Tb, background=100, gls=True)
    t0 = time.perf_counter()
    batch = engine.Batch(cfgs, lanes=1)
    outs = batch.alloc_device_outputs()
    lane_ms = batch.autotune(stack, outs, max_lanes=4)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    batch.execute(stack, outs)                  # capture (after the tuner's last assignment)
    batch.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = max(3, steps)
    e0.record(stream)
    for _ in range(n):
        batch.execute(stack, outs)
    e1.record(stream)
    batch.synchronize()
    graph_ms = e0.elapsed_time(e1) / n
    npix = sum(c.npix for c in cfgs)
    fitted = sum(int(o["fitted"].sum().item()) for o in outs)
    infos = [batch.job_info(i) for i in range(len(cfgs))]
    # without the graph: the jobs' own times, each executed alone (eager
    # launches on one stream, measured by the autotuner)
    seq_ms = sum(i["ms"] for i in infos)
    # bitwise equality of three jobs with standalone plans (same tiles)
    checked = equal = 0
    for k in (0, len(cfgs) // 2, len(cfgs) - 1):
        p = engine.Plan(cfgs[k])
        p.set_corr_tile(infos[k]["cta"], infos[k]["seg_extra"], infos[k]["tail_extra"])
        o = p.alloc_device_outputs()
        p.execute(stack, o)
        p.synchronize()
        checked += 1
        equal += int(all(torch.equal(torch.isnan(o[nm]), torch.isnan(outs[k][nm])) and
                         torch.equal(o[nm].nan_to_num(0.0), outs[k][nm].nan_to_num(0.0)) if o[nm].is_floating_point()
                         else torch.equal(o[nm], outs[k][nm]) for nm in o))
        p.close()
        del o
    tiles = {}
    for i in infos:
        key = f"{i['cta']}x2^{i['seg_extra']}/2^{i['tail_extra']}"
        tiles[key] = tiles.get(key, 0) + 1
    blk = {"workload": f"{Wb}x{Hb}x{Tb} uint16 (GPU Monte-Carlo, D1 0.5 / D2 5 um^2/s, 70/30); binnings 1-5 x "
                       "offsets {0,1,2}^2 = 45 jobs; GLS covariance + GLS LM fit (N, D, G)",
           "jobs": len(cfgs), "pixels": npix, "fitted": fitted, "graph_ms": graph_ms,
           "pixels_per_s": npix / (graph_ms * 1e-3), "jobs_alone_sum_ms": seq_ms,
           "graph_speedup_vs_jobs_alone": seq_ms / graph_ms, "lanes": batch.lanes, "lane_ms": lane_ms,
           "gpu_launches_per_graph": batch.kernel_launches(), "tiles": tiles,
           "scratch_gb": batch.scratch_bytes / 1e9, "simulate_s": sim_s, "create_and_autotune_s": tune_s,
           "bitwise_equal_standalone": f"{equal}/{checked}"}
    batch.close()
    return blk


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from imaging_fcs_1_52_gb300 import _lib, engine

    cfg = make_config(engine, _lib)
    stack_np = host_stack(seed=1 + rank)                # each rank: its own stack (weak scaling)
    stack = torch.from_numpy(stack_np.view(np.int16)).cuda().view(torch.uint16)
    torch.cuda.synchronize()
    plan = engine.Plan(cfg)
    out = plan.alloc_device_outputs()
    stream = torch.cuda.current_stream()
    # the correlator tile, chosen by the autotuner on this stack (untimed)
    tile_trials = plan.autotune(stack, out)
    tile_chosen = dict(zip(("cta", "seg_extra", "tail_extra"), plan.corr_tile()))
    plan.set_timing(True)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        plan.execute(stack, out)
    barrier()
    corr_ms = []
    launches = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the timed steps sit in an NVTX range ("timed"), so that a profiler can
    # select exactly them (ncu --nvtx --nvtx-include timed/)
    with ClockSampler(local) as clk, torch.cuda.nvtx.range("timed"):
        e0.record(stream)
        stage_acc = None
        for _ in range(args.steps):
            plan.execute(stack, out)
            launches += plan.kernel_launches()
            torch.cuda.synchronize()     # stage events of this step are then readable
            st = plan.stage_times()
            # the correlator path from the raw stack to G and variance: the
            # streaming pass, the blocking transform and the level chain
            corr_ms.append(st["stream"] + st["blocking"] + st["correlator"])
            stage_acc = st if stage_acc is None else {k: stage_acc[k] + st[k] for k in st}
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * cfg.npix / (ms * 1e-3)

    # e2e through the C ABI with host buffers (pinned host stack)
    host = torch.empty((T, H, W), dtype=torch.int16, pin_memory=True)
    host.copy_(torch.from_numpy(stack_np.view(np.int16)))
    host_np = host.numpy().view(np.uint16)
    # results land in pinned host buffers (page-locked, as the stack): the
    # device-to-host copies then run at link speed instead of through a
    # pageable bounce buffer
    outs_host = {}
    tdt = {"f8": torch.float64, "f4": torch.float32, "i4": torch.int32}
    for n in engine.output_names(cfg):
        dt, shp = engine._OUT_SPEC[n]
        outs_host[n] = torch.empty((cfg.npix, *shp(cfg.chanum)), dtype=tdt[dt], pin_memory=True).numpy()
    plan.execute_host(host_np, outs_host)           # warm-up of the host path
    barrier()
    # every step copies its stack in and its results out; through the
    # asynchronous entry the next step's stack copy overlaps this step's
    # execution (two device stack buffers used in turn)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plan.execute_host_async(host_np, outs_host)
    plan.synchronize()
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    h2d = T * H * W * 2
    d2h = sum(v.nbytes for v in outs_host.values())

    if rank == 0:
        peak, peak_kind = measured_peaks()
        corr_avg = statistics.mean(corr_ms)
        # algorithmic bytes of the correlator path: the uint16 stack once +
        # ACF and blocked variance out (8 B each per pixel and channel)
        alg_bytes = T * H * W * 2 + cfg.npix * cfg.chanum * 8 * 2
        achieved = alg_bytes / (corr_avg * 1e-3) / 1e9
        sample = args.cpu_sample or 4096
        cpu_v, cpu_n, cpu_dt, ref = cpu_baseline(stack_np, cfg, sample, os.cpu_count() or 1)
        # single-threaded, as the plugin's one worker thread runs it
        cpu1_v, cpu1_n, cpu1_dt, _ = cpu_baseline(stack_np, cfg, min(sample, 256), 1)
        gpu_np = {k: v.cpu().numpy() for k, v in out.items()}
        parity = parity_block(gpu_np, ref, cpu_n)
        if cfg.bleach in (_lib.BLEACH_SINGLE_EXP, _lib.BLEACH_DOUBLE_EXP):
            # pixels whose exponential bleach rate the averaged trace does not
            # determine (standard error >= the rate: a decay faster than the
            # first averaged point, or a curve in the tau -> infinity valley):
            # their least-squares minimum is flat along a curve, so the
            # correction depends on where an optimiser stops
            import oracle
            ncols = min(cpu_n, W)
            det = oracle.bleach_rate_determined(np.ascontiguousarray(stack_np[:, :cpu_n // ncols, :ncols]), ncols,
                                                cpu_n // ncols, background=cfg.background, frametime=cfg.frametime,
                                                two=cfg.bleach == _lib.BLEACH_DOUBLE_EXP)
            parity["bleach_rate_undetermined"] = int((~det).sum())
            parity["determined"] = parity_block(gpu_np, ref, cpu_n, det)
        fitted = int(out["fitted"].sum().item())
        try:
            rooflines = compute_rooflines(_lib.load(), cfg, stage_acc["fits"] / args.steps,
                                          int(out["iterations"].sum().item()))
        except Exception as e:   # reported, never fatal to the bench line
            rooflines = {"error": str(e)}
        sur_blk = surrogate_block(plan, stack, args.steps)
        bands_blk = (bands_block(engine, cfg, host_np, outs_host, plan.corr_tile(), min(args.steps, 5))
                     if world == 1 else None)
        batch_blk = None
        if not args.no_batch and world == 1:
            plan.close()
            del out, stack
            torch.cuda.empty_cache()
            batch_blk = batch_block(args.steps)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (tests/synth_host.c, seeded; same stack as the reference arm)",
            "config": {"workload": f"128x128x{T} uint16 stack; single-exp bleach; P=16 Q=8 (73 ch); "
                                   "blocked variance; OLS LM TIRF fit (N, D, G)",
                       "pixels_per_rank": cfg.npix, "frames": T, "l2": f"stack {T * H * W * 2 / 1e9:.2f} GB > L2 (129 MB), no flush needed",
                       "parallelism": f"pixel shards x{world}", "fitted_pixels": fitted},
            "fitted_pixels_per_s": world * fitted / (ms * 1e-3),
            "e2e": {"value": world * cfg.npix / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "gpu_launches": launches,
            "stages_ms": {k: v / args.steps for k, v in stage_acc.items()},
            "corr_tile": {"chosen": tile_chosen, "trials": tile_trials},
            "roofline": {"kernel": "correlator path: stream_tma (values + monitors), monitor_finalize, block, "
                                   "block_finalize, c2_pair x2, c2_tail, c2_finalize",
                         "bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": load_profile_traffic(),
                         "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": corr_avg},
            "rooflines_other": rooflines,
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"{cpu_n} pixels x {T} frames of the same stack, FP64 C oracle, "
                                       f"{cpu_dt:.1f} s"},
            "cpu_baseline_single_thread": {"value": cpu1_v, "unit": UNIT, "cores": 1, "kind": "port",
                                           "sample": f"{cpu1_n} pixels x {T} frames, {cpu1_dt:.1f} s"},
            "clocks": clk.summary(),
            "parity": parity,
            "surrogate": sur_blk,
            "bands": bands_blk,
            "batch_config3": batch_blk,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
