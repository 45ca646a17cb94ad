"""Learned LM seeds: the MLP surrogate of the fit (imfcs_surrogate_*).

No counterpart in the reference: every fit of the plugin starts from the
configured initial values (Imaging_FCS_1_52.java:1958-1970, handed to the
GPU fit at java:15112-15185).  Here a small network maps a pixel's
normalised ACF and its standard deviation (lags 1..64) to standardised
predictions of

    log D [um^2/s],  log(N G(1)),  G_inf / G(1),  fraction of a 2nd component

and a plan with the surrogate attached (Plan.set_surrogate) starts each
pixel's LM from them.  Plain LM from the configured initial values stays the
fallback (failed seeded fits are refit) and, in mode 2, the arbiter.

Training data come from the project's own Monte-Carlo simulator
(imfcs_simulate) and correlator: seeded stacks over log-uniform D, N and
frame counts, each correlated and fitted by plain LM through a Plan; the
network learns to predict where plain LM ends (log D, log N G(1), G / G(1))
and the simulated second-component fraction.  Training and inference run
the library's BF16 tensor-core kernels with FP32 accumulation and FP32
Adam master weights.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os

import numpy as np

from . import _lib
from ._lib import check

N_IN, N_HID, N_OUT = 128, 256, 4
N_LAGS = 64
TARGETS = ("log_D_um2_s", "log_N_G1", "G_inf_over_G1", "fraction2")

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "data", "surrogate_tirf_1ms.npz")


def param_layout() -> dict:
    """Offsets and shapes of the flat FP32 parameter vector."""
    shapes = [("W1", (N_IN, N_HID)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
              ("W3", (N_HID, N_OUT)), ("b3", (N_OUT,))]
    out, off = {}, 0
    for name, shp in shapes:
        n = int(np.prod(shp))
        out[name] = (off, shp)
        off += n
    return out


def split_params(flat: np.ndarray) -> dict:
    """Views of the network blocks plus the target standardisation."""
    lay = param_layout()
    d = {k: flat[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}
    p = sum(int(np.prod(s)) for _, s in lay.values())
    d["tmean"] = flat[p:p + N_OUT]
    d["tstd"] = flat[p + N_OUT:p + 2 * N_OUT]
    return d


class Surrogate:
    """A device-resident MLP (imfcs_surrogate handle)."""

    def __init__(self, seed: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        check(self._L.imfcs_surrogate_create(C.c_uint64(seed), C.byref(h)), "imfcs_surrogate_create")
        self._h = h
        self.meta: dict = {}

    @property
    def handle(self):
        return self._h

    @property
    def param_count(self) -> int:
        return int(self._L.imfcs_surrogate_param_count())

    def close(self):
        if getattr(self, "_h", None):
            self._L.imfcs_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters -------------------------------------------------------
    def params(self) -> np.ndarray:
        out = np.empty(self.param_count + 2 * N_OUT, np.float32)
        check(self._L.imfcs_surrogate_get_params(self._h, C.c_void_p(out.ctypes.data)), "imfcs_surrogate_get_params")
        return out

    def set_params(self, flat: np.ndarray) -> None:
        flat = np.ascontiguousarray(flat, np.float32)
        if flat.size != self.param_count + 2 * N_OUT:
            raise ValueError(f"expected {self.param_count + 2 * N_OUT} values, got {flat.size}")
        check(self._L.imfcs_surrogate_set_params(self._h, C.c_void_p(flat.ctypes.data)), "imfcs_surrogate_set_params")

    def save(self, path: str, **meta) -> None:
        m = dict(self.meta)
        m.update(meta)
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, params=self.params(), meta=np.array(json.dumps(m)))

    @classmethod
    def load(cls, path: str = DEFAULT_WEIGHTS) -> "Surrogate":
        z = np.load(path)
        s = cls(0)
        s.set_params(z["params"])
        s.meta = json.loads(str(z["meta"]))
        return s

    # -- device compute ------------------------------------------------------
    def features(self, acf, var):
        """CUDA float64 acf/var [npix][chanum] -> CUDA float32 [npix][128]."""
        import torch
        assert acf.is_cuda and acf.dtype == torch.float64 and acf.is_contiguous()
        assert var.is_cuda and var.dtype == torch.float64 and var.is_contiguous()
        npix, chanum = acf.shape
        x = torch.empty((npix, N_IN), dtype=torch.float32, device=acf.device)
        st = torch.cuda.current_stream()
        check(self._L.imfcs_surrogate_features(npix, chanum, C.c_void_p(acf.data_ptr()), C.c_void_p(var.data_ptr()),
                                               C.c_void_p(x.data_ptr()), C.c_void_p(st.cuda_stream)),
              "imfcs_surrogate_features")
        return x

    def gradients(self, x, t):
        """Mean-squared-error gradients (flat FP32, host) and loss on one batch
        (targets standardised by the current mean / std)."""
        import torch
        x = x.contiguous().float()
        t = t.contiguous().float()
        assert x.is_cuda and t.is_cuda and x.shape[1] == N_IN and t.shape[1] == N_OUT
        torch.cuda.synchronize()
        g = np.empty(self.param_count, np.float32)
        loss = C.c_double()
        check(self._L.imfcs_surrogate_gradients(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                                x.shape[0], C.c_void_p(g.ctypes.data), C.byref(loss)),
              "imfcs_surrogate_gradients")
        return g, float(loss.value)

    def train(self, x, t, steps: int, batch: int = 1024, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        """Adam on (x, t) (CUDA float32, rows already shuffled); returns the
        per-step minibatch losses (standardised units)."""
        import torch
        x = x.contiguous().float()
        t = t.contiguous().float()
        hist = np.empty(steps, np.float32)
        st = torch.cuda.current_stream()
        check(self._L.imfcs_surrogate_train(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                            x.shape[0], int(steps), int(batch), C.c_float(lr), C.c_uint64(seed),
                                            C.c_void_p(hist.ctypes.data), C.c_void_p(st.cuda_stream)),
              "imfcs_surrogate_train")
        return hist

    def predict(self, x):
        """CUDA float32 [n][128] -> de-standardised predictions [n][4]."""
        import torch
        x = x.contiguous().float()
        out = torch.empty((x.shape[0], N_OUT), dtype=torch.float32, device=x.device)
        st = torch.cuda.current_stream()
        check(self._L.imfcs_surrogate_predict(self._h, C.c_void_p(x.data_ptr()), x.shape[0],
                                              C.c_void_p(out.data_ptr()), C.c_void_p(st.cuda_stream)),
              "imfcs_surrogate_predict")
        return out


# ---------------------------------------------------------------------------
# Training data: simulator + correlator + plain LM.
# ---------------------------------------------------------------------------
PIXEL_UM, PSF_UM, FRAMETIME = 0.24, 0.4, 1e-3


def obs_area_um2(pixel_um: float = PIXEL_UM, psf_um: float = PSF_UM) -> float:
    """Observation area of the TIRF model for one pixel (um^2): N = density x area."""
    from .engine import obsvol_2d
    return obsvol_2d(pixel_um * 1e-6, pixel_um * 1e-6, psf_um * 1e-6) * 1e12


def fit_config(side: int, frames: int, *, bleach: int | None = None, q: int = 8):
    """The plain-LM configuration the surrogate is trained for and used with:
    P=16, 1 ms frames, 0.24 um pixels, PSF 0.4 um, single-exponential bleach
    correction, OLS LM of N, D, G from the default initial values."""
    from . import engine
    return engine.FCSConfig(width=side, height=side, frames=frames, background=100,
                            bleach=_lib.BLEACH_SINGLE_EXP if bleach is None else bleach, p=16, q=q,
                            frametime=FRAMETIME, do_fit=True)


def sample_stack_params(rng: np.random.Generator, d_range=(0.05, 20.0), n_range=(0.2, 200.0),
                        frame_range=(10000, 100000), two_comp_prob=0.2):
    """One training stack's draw: log-uniform density (from N), frame count,
    a per-16x16-tile D map (log-uniform) or, for a two-component stack, a
    global (D1, D2 = D1 / r, fraction) with r in [3, 30]; a bleach time
    constant log-uniform in 5..200 s for half of the stacks."""
    lo, hi = np.log(d_range)
    n_target = float(np.exp(rng.uniform(*np.log(n_range))))
    frames = int(np.exp(rng.uniform(*np.log(frame_range))))
    p = {"density": n_target / obs_area_um2(), "n_target": n_target, "frames": frames,
         "tau_bleach": float(np.exp(rng.uniform(np.log(5.0), np.log(200.0)))) if rng.random() < 0.5 else 0.0}
    if rng.random() < two_comp_prob:
        d1 = float(np.exp(rng.uniform(lo, hi)))
        p.update(two=True, d1=d1, d2=d1 / float(rng.uniform(3.0, 30.0)), fraction2=float(rng.uniform(0.1, 0.9)))
    else:
        p.update(two=False, d1=1.0, d2=0.0, fraction2=0.0)
    p["dlog"] = (float(lo), float(hi))
    return p


def simulate_training_stack(p: dict, side: int, seed: int):
    """CUDA uint16 stack [frames][side][side] for one draw of sample_stack_params."""
    from . import engine
    dmap = None
    if not p["two"]:
        rng = np.random.default_rng(seed)
        nt = (side + 15) // 16
        dmap = np.exp(rng.uniform(*p["dlog"], (nt, nt))).astype(np.float32)
    return engine.simulate(side, side, p["frames"], density=p["density"], d1=p["d1"], d2=p["d2"],
                           fraction2=p["fraction2"], tau_bleach=p["tau_bleach"], steps_per_frame=4,
                           pixel_um=PIXEL_UM, psf_um=PSF_UM, seed=seed, d_tile_map=dmap)


def targets_from_fit(acf, fitres, fitted, fraction2: float):
    """Targets [n][4] on the device for the fitted pixels, and their mask."""
    import torch
    g1 = acf[:, 1]
    n = fitres[:, 0].double()
    d = fitres[:, 1].double() * 1e12
    g = fitres[:, 4].double()
    ok = (fitted != 0) & torch.isfinite(g1) & (g1 > 0) & (n > 0) & (d > 0) & torch.isfinite(g)
    t = torch.stack([torch.log(d.clamp_min(1e-30)), torch.log((n * g1).clamp_min(1e-30)), g / g1,
                     torch.full_like(g1, fraction2)], dim=1).float()
    ok &= torch.isfinite(t).all(dim=1)
    return t, ok


def make_training_set(n_curves: int, *, side: int = 64, seed: int = 1, q: int = 8, log=None,
                      max_seconds: float = 0.0, **draw):
    """Simulate + correlate + plain-LM-fit stacks until n_curves usable curves
    (or max_seconds > 0 has passed): returns CUDA float32 x [n][128], t [n][4]
    (shuffled) and a summary.  The N range of the draw (default 0.2-200)
    covers 0.5-200 and the sparse bench stacks (N ~ 0.3)."""
    import time

    import torch
    from . import engine
    rng = np.random.default_rng(seed)
    xs, ts, n, stacks, sim_s = [], [], 0, 0, 0.0
    sur = Surrogate(0)   # features only
    start = time.perf_counter()
    while n < n_curves and not (max_seconds > 0 and time.perf_counter() - start > max_seconds and n > 0):
        p = sample_stack_params(rng, **draw)
        stack_side = side if not p["two"] else max(16, side // 2)
        t0 = time.perf_counter()
        st = simulate_training_stack(p, stack_side, seed * 100003 + stacks)
        torch.cuda.synchronize()
        sim_s += time.perf_counter() - t0
        cfg = fit_config(stack_side, p["frames"], q=q)
        plan = engine.Plan(cfg)
        try:
            out = plan.alloc_device_outputs()
            plan.execute(st, out)
            x = sur.features(out["acf"], out["var"])
            t, ok = targets_from_fit(out["acf"], out["fitres"], out["fitted"], p["fraction2"])
        finally:
            plan.close()
        del st
        xs.append(x[ok])
        ts.append(t[ok])
        n += int(ok.sum())
        stacks += 1
        if log:
            log(f"stack {stacks}: {stack_side}^2 x {p['frames']} N~{p['n_target']:.2f} two={p['two']} "
                f"usable {int(ok.sum())} total {n}")
    sur.close()
    x = torch.cat(xs)[:n_curves]
    t = torch.cat(ts)[:n_curves]
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    perm = torch.randperm(x.shape[0], generator=g).to(x.device)
    info = {"curves": int(x.shape[0]), "stacks": stacks, "side": side, "simulate_s": round(sim_s, 2),
            "q": q, "draw": {k: (list(v) if isinstance(v, tuple) else v) for k, v in draw.items()}}
    return x[perm].contiguous(), t[perm].contiguous(), info


def train_surrogate(x, t, *, epochs: float = 20.0, batch: int = 1024, lr: float = 1e-3, seed: int = 0,
                    log=None) -> tuple[Surrogate, dict]:
    """Train a new surrogate on (x, t): Adam with a cosine learning-rate decay
    applied in 20 segments; returns the surrogate and a training summary."""
    n = x.shape[0]
    steps = max(1, int(round(epochs * n / batch)))
    sur = Surrogate(seed)
    segs = 20
    hist = []
    done = 0
    for i in range(segs):
        k = steps * (i + 1) // segs - done
        if k <= 0:
            continue
        lr_i = lr * 0.5 * (1 + math.cos(math.pi * (i + 0.5) / segs)) + lr * 0.01
        h = sur.train(x, t, k, batch=batch, lr=lr_i, seed=seed * 7919 + i)
        hist.append(h)
        done += k
        if log:
            log(f"segment {i + 1}/{segs}: steps {done}, lr {lr_i:.2e}, loss {float(h[-min(50, len(h)):].mean()):.4f}")
    hist = np.concatenate(hist)
    info = {"steps": steps, "batch": batch, "lr": lr, "epochs": epochs,
            "loss_first": float(hist[:20].mean()), "loss_last": float(hist[-200:].mean())}
    sur.meta.update(train=info)
    return sur, info
