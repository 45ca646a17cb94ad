"""Train the fit surrogate on the GPU and save its weights.

    python -m imaging_fcs_1_52_gb300.train_surrogate --curves 1000000 \
        --out imaging_fcs_1_52_gb300/data/surrogate_tirf_1ms.npz

Curves: seeded Monte-Carlo stacks (imfcs_simulate) over log-uniform D,
density and frame counts, correlated and fitted by plain LM through a Plan
(surrogate.make_training_set); 2 % are held out.  Training: the library's
BF16 tensor-core forward/backward kernels with Adam (surrogate.train_surrogate).
The weights file records the optical and correlator configuration it was
trained for, the data draw and the losses.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--curves", type=int, default=1_000_000)
    ap.add_argument("--side", type=int, default=64)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--epochs", type=float, default=8.0)
    ap.add_argument("--batch", type=int, default=2048)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--n-min", type=float, default=0.2)
    ap.add_argument("--n-max", type=float, default=200.0)
    ap.add_argument("--max-sim-seconds", type=float, default=0.0, help="stop generating after this long (0 = no limit)")
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)

    import torch
    from . import surrogate

    t0 = time.perf_counter()
    log = lambda m: print(f"[{time.perf_counter() - t0:8.1f}s] {m}", flush=True)
    x, t, info = surrogate.make_training_set(a.curves, side=a.side, seed=a.seed, log=log,
                                             n_range=(a.n_min, a.n_max), max_seconds=a.max_sim_seconds)
    gen_s = time.perf_counter() - t0
    n = x.shape[0]
    nh = max(1, n // 50)
    xh, th = x[:nh], t[:nh]
    xt, tt = x[nh:], t[nh:]
    log(f"data: {n} curves from {info['stacks']} stacks in {gen_s:.1f} s; training on {xt.shape[0]}")
    t1 = time.perf_counter()
    sur, tr = surrogate.train_surrogate(xt, tt, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, log=log)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    p = sur.predict(xh).cpu().numpy()
    th_np = th.cpu().numpy()
    hold = {name: {"rmse": float(np.sqrt(np.mean((p[:, i] - th_np[:, i]) ** 2))),
                   "target_sd": float(th_np[:, i].std())}
            for i, name in enumerate(surrogate.TARGETS)}
    log(f"trained {tr['steps']} steps in {train_s:.1f} s; held-out: {json.dumps(hold)}")
    sur.save(a.out, config={"p": 16, "q": info["q"], "frametime_s": surrogate.FRAMETIME,
                            "pixel_um": surrogate.PIXEL_UM, "psf_um": surrogate.PSF_UM,
                            "model": "TIRF FCS_3p, 1 component, N D G free, OLS",
                            "bleach": "single exponential"},
             data=info, train=dict(tr, seconds=round(train_s, 2)), holdout=hold,
             generate_seconds=round(gen_s, 2))
    log(f"saved {a.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
