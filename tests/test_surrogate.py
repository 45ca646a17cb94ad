"""The learned part: MLP surrogate kernels (BF16 tensor cores, FP32
accumulation) against torch-CPU FP64 autograd, its training on simulator +
correlator curves, and surrogate-seeded LM against plain LM (the arbiter).

Also the simulator check the training data rest on: correlate + fit of a
simulated stack recovers the simulated D and N (the semantics of
simulateACF2D, Imaging_FCS_1_52.java:13854-14409, with the TIRF model of
java:13135-13145)."""
import numpy as np
import pytest

from imaging_fcs_1_52_gb300 import _lib, engine, surrogate

# ---------------------------------------------------------------------------
# CPU: layout of the parameter vector.
# ---------------------------------------------------------------------------


def test_param_layout_matches_library():
    L = _lib.load()
    lay = surrogate.param_layout()
    total = sum(int(np.prod(s)) for _, s in lay.values())
    assert total == int(L.imfcs_surrogate_param_count()) == 128 * 256 + 256 + 256 * 256 + 256 + 256 * 4 + 4
    flat = np.arange(total + 8, dtype=np.float32)
    d = surrogate.split_params(flat)
    assert d["W1"].shape == (128, 256) and d["W3"].shape == (256, 4)
    assert d["tmean"][0] == total and d["tstd"][-1] == total + 7


def test_obs_area_and_density():
    # N = density x observation area; 0.24 um pixels, 0.4 um PSF radius
    a = surrogate.obs_area_um2()
    assert 0.4 < a < 0.7


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------


def _torch_reference(flat, x, t, emulate_bf16):
    """Forward + MSE + backward in FP64 (torch CPU autograd).  With
    emulate_bf16 the operands are rounded to BF16 where the kernels round
    them (inputs, weights, hidden activations, back-propagated deltas)."""
    import torch
    d = surrogate.split_params(flat.astype(np.float64))
    P = {k: torch.tensor(np.array(v), dtype=torch.float64, requires_grad=True)
         for k, v in d.items() if k not in ("tmean", "tstd")}

    class BF(torch.autograd.Function):
        # an activation stored as BF16 (its gradient passes through unrounded)
        @staticmethod
        def forward(ctx, a):
            return a.to(torch.bfloat16).to(torch.float64) if emulate_bf16 else a

        @staticmethod
        def backward(ctx, g):
            return g

    def bw(w):   # weight used as a BF16 operand (gradient stays in full precision)
        return w + (w.detach().to(torch.bfloat16).to(torch.float64) - w.detach()) if emulate_bf16 else w

    def gelu(z):
        return 0.5 * z * (1 + torch.erf(z / np.sqrt(2.0)))

    class GradRound(torch.autograd.Function):
        # identity forward; the gradient flowing back is rounded to BF16
        @staticmethod
        def forward(ctx, a):
            return a

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).to(torch.float64) if emulate_bf16 else g

    X = torch.tensor(x, dtype=torch.float64)
    if emulate_bf16:
        X = X.to(torch.bfloat16).to(torch.float64)
    T = torch.tensor(t, dtype=torch.float64)
    z1 = X @ bw(P["W1"]) + P["b1"]
    h1 = BF.apply(gelu(GradRound.apply(z1)))
    z2 = h1 @ bw(P["W2"]) + P["b2"]
    h2 = BF.apply(gelu(GradRound.apply(z2)))
    y = GradRound.apply(h2 @ bw(P["W3"]) + P["b3"])
    loss = ((y - T) ** 2).mean()
    loss.backward()
    g = np.concatenate([P[k].grad.numpy().ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3")])
    return g, float(loss)


@pytest.mark.gpu
def test_gradients_match_fp64_autograd():
    """Forward + backward kernels against FP64 autograd: with BF16 rounding
    emulated at the kernels' rounding points the gradients agree to the FP32
    accumulation level; against plain FP64 they agree to BF16 precision."""
    import torch
    rng = np.random.default_rng(5)
    n = 300   # not a multiple of the 64-row tiles
    sur = surrogate.Surrogate(seed=3)
    flat = sur.params()
    d = surrogate.split_params(flat)
    d["b1"][:] = rng.normal(0, 0.1, d["b1"].shape)
    d["b2"][:] = rng.normal(0, 0.1, d["b2"].shape)
    d["b3"][:] = rng.normal(0, 0.1, d["b3"].shape)
    d["tmean"][:] = 0.0
    d["tstd"][:] = 1.0
    sur.set_params(flat)
    x = rng.normal(0, 1, (n, 128)).astype(np.float32)
    t = rng.normal(0, 1, (n, 4)).astype(np.float32)
    g, loss = sur.gradients(torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda"))
    ge, le = _torch_reference(flat, x, t, emulate_bf16=True)
    gf, lf = _torch_reference(flat, x, t, emulate_bf16=False)
    assert abs(loss - le) <= 1e-3 * abs(le)
    assert abs(loss - lf) <= 2e-2 * abs(lf)
    lay = surrogate.param_layout()
    for k, (o, shp) in lay.items():
        m = int(np.prod(shp))
        a, e, f = g[o:o + m], ge[o:o + m], gf[o:o + m]
        rel_e = np.linalg.norm(a - e) / np.linalg.norm(e)
        rel_f = np.linalg.norm(a - f) / np.linalg.norm(f)
        assert rel_e <= 1e-2, (k, rel_e)
        assert rel_f <= 5e-2, (k, rel_f)


@pytest.mark.gpu
def test_features_from_correlator_outputs():
    import torch
    rng = np.random.default_rng(2)
    npix, chanum = 37, 73
    acf = rng.normal(0, 0.1, (npix, chanum))
    acf[:, 1] = rng.uniform(0.05, 2.0, npix)
    acf[3, 1] = 0.0                         # G(1) = 0: non-finite ratios -> 0
    var = rng.uniform(1e-6, 1e-2, (npix, chanum))
    var[5, 10] = np.nan
    sur = surrogate.Surrogate(0)
    x = sur.features(torch.tensor(acf, device="cuda"), torch.tensor(var, device="cuda")).cpu().numpy()
    with np.errstate(divide="ignore", invalid="ignore"):
        g = acf[:, 1:65] / acf[:, 1:2]
        s = np.sqrt(var[:, 1:65]) / np.abs(acf[:, 1:2])
    g = np.where(np.isfinite(g), np.clip(g, -8, 8), 0.0)
    s = np.where(np.isfinite(s), np.minimum(s, 8), 0.0)
    ref = np.concatenate([g, s], axis=1)
    np.testing.assert_allclose(x, ref, rtol=1e-6, atol=1e-7)


@pytest.mark.gpu
def test_simulator_recovers_d_and_n():
    """Correlate + fit of a simulated stack gives back the simulated D and N
    (N = density x observation area of the TIRF model): medians over 48 x 48
    pixels of 50,000 frames within 6 % (the spread between seeds of the same
    draw is about 2 %; 24 x 24 x 20,000 stacks scatter by 5-10 %)."""
    for d_sim, density in ((1.0, 2.0), (5.0, 8.0)):
        st = engine.simulate(48, 48, 50000, d1=d_sim, density=density, steps_per_frame=10, seed=11)
        cfg = surrogate.fit_config(48, 50000, bleach=_lib.BLEACH_NONE)
        plan = engine.Plan(cfg)
        out = plan.alloc_device_outputs()
        plan.execute(st, out)
        fr = out["fitres"].cpu().numpy()
        ok = out["fitted"].cpu().numpy() == 1
        plan.close()
        assert ok.mean() > 0.95
        d_med = np.median(fr[ok, 1]) * 1e12
        n_med = np.median(fr[ok, 0])
        n_sim = density * surrogate.obs_area_um2()
        assert abs(d_med / d_sim - 1) < 0.06, (d_sim, d_med)
        assert abs(n_med / n_sim - 1) < 0.06, (n_sim, n_med)


_TRAINED = {}


def _trained_surrogate():
    """The committed weights when present, else a small network trained
    here on simulator + correlator curves."""
    import os
    if "s" not in _TRAINED:
        if os.path.exists(surrogate.DEFAULT_WEIGHTS):
            _TRAINED["s"] = surrogate.Surrogate.load()
        else:
            x, t, _ = surrogate.make_training_set(24000, side=32, seed=3, frame_range=(10000, 30000))
            _TRAINED["s"], _ = surrogate.train_surrogate(x, t, epochs=30, batch=512, lr=2e-3)
    return _TRAINED["s"]


@pytest.mark.gpu
def test_training_reduces_loss_on_simulated_curves():
    import torch
    x, t, info = surrogate.make_training_set(3000, side=32, seed=9, frame_range=(10000, 20000))
    assert x.shape == (3000, 128) and t.shape == (3000, 4)
    assert torch.isfinite(x).all() and torch.isfinite(t).all()
    sur, tr = surrogate.train_surrogate(x[:2500], t[:2500], epochs=40, batch=256, lr=2e-3)
    assert tr["loss_last"] < 0.5 * tr["loss_first"]
    # held-out curves: the predicted log D beats the training mean
    p = sur.predict(x[2500:]).cpu().numpy()
    tt = t[2500:].cpu().numpy()
    mse_pred = np.mean((p[:, 0] - tt[:, 0]) ** 2)
    mse_mean = np.mean((tt[:, 0] - tt[:2500, 0].mean()) ** 2) if len(tt) > 1 else 1.0
    assert mse_pred < 0.5 * np.var(tt[:, 0]) + 1e-12, (mse_pred, mse_mean)


def _fresh_stack():
    rng = np.random.default_rng(77)
    dmap = np.exp(rng.uniform(np.log(0.2), np.log(10.0), (4, 4))).astype(np.float32)
    return engine.simulate(64, 64, 20000, density=2.0, tau_bleach=20.0, seed=4242, d_tile_map=dmap)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_seeded_fit_matches_plain(mode):
    """Surrogate-seeded LM reaches the plain-LM chi^2 (within 1 %) and the
    same N and D on a fresh simulated stack, in fewer LM iterations."""
    sur = _trained_surrogate()
    st = _fresh_stack()
    cfg = surrogate.fit_config(64, 20000)
    plan = engine.Plan(cfg)
    ref = plan.alloc_device_outputs()
    plan.execute(st, ref)
    out = plan.alloc_device_outputs()
    plan.set_surrogate(sur, mode)
    plan.execute(st, out)
    stats = plan.surrogate_stats()
    plan.close()
    r = {k: v.cpu().numpy() for k, v in ref.items()}
    o = {k: v.cpu().numpy() for k, v in out.items()}
    np.testing.assert_array_equal(o["acf"], r["acf"])
    both = (r["fitted"] == 1) & (o["fitted"] == 1)
    assert (r["fitted"] == o["fitted"]).mean() >= 0.99
    assert both.sum() > 3000
    chi_ratio = o["chi2"][both] / r["chi2"][both]
    assert (chi_ratio <= 1.01).mean() >= 0.99
    if mode == 2:
        assert (chi_ratio <= 1.01 + 1e-6).all()
    for i in (0, 1):
        rel = np.abs(o["fitres"][both, i] / r["fitres"][both, i] - 1)
        assert (rel <= 1e-3).mean() >= 0.99, (i, np.quantile(rel, 0.99))
    assert stats["refit"] < 0.10 * cfg.npix
    assert o["iterations"].mean() < r["iterations"].mean()


@pytest.mark.gpu
def test_set_surrogate_rejects_bad_use():
    sur = surrogate.Surrogate(0)
    cfg = surrogate.fit_config(16, 4000)
    cfg.do_fit = False
    plan = engine.Plan(cfg)
    with pytest.raises(_lib.ImfcsError):
        plan.set_surrogate(sur, 1)
    plan.close()
    plan = engine.Plan(surrogate.fit_config(16, 4000))
    with pytest.raises(_lib.ImfcsError):
        plan.set_surrogate(sur, 3)
    plan.set_surrogate(sur, 1)
    plan.set_surrogate(None)
    plan.close()
