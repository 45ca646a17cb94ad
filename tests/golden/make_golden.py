"""Generates tests/golden/*.npz: oracle (FP64) outputs on seeded synthetic
stacks.  `config1_poly4` has the shape of the reference plugin's CPU-runnable
workload (21 x 21 pixels x 20,000 frames of 1 ms, polynomial bleach
correction of order 4, P=16 Q=8, one-component TIRF fit of N, D, G);
`bright_ccf_bin2` covers binning, cross-correlation and the single
exponential bleach correction.  Stacks are regenerated from their seeds
(tests/synth.py); the file stores the stack's checksum so a change of the
generator is detected instead of silently compared.

The reference ships no golden vectors and its Java path cannot run here, so
these fixtures pin the oracle against itself (regression) and give the GPU
tests fixed expected values; they do not pin the oracle to the Java code.

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from imaging_fcs_1_52_gb300 import engine  # noqa: E402
from tests.helpers import oracle_kwargs  # noqa: E402
from tests.synth import brownian_stack  # noqa: E402

CASES = {
    # name: (stack kwargs, FCSConfig kwargs without width/height/frames)
    "config1_poly4": (dict(width=21, height=21, frames=20000, seed=1),
                      dict(background=100, bleach=oracle.BLEACH_POLY, poly_order=4)),
    "bright_ccf_bin2": (dict(width=10, height=9, frames=6000, seed=7, density=2.0, cps=30000.0, tau_bleach=8.0),
                        dict(background=100, binx=2, biny=2, cfx=1, cfy=1, bleach=oracle.BLEACH_SINGLE_EXP)),
}


def case_config(name):
    skw, ckw = CASES[name]
    cst = engine.model_constants(binx=ckw.get("binx", 1), biny=ckw.get("biny", 1), cfx=ckw.get("cfx", 0),
                                 cfy=ckw.get("cfy", 0))
    return skw, engine.FCSConfig(width=skw["width"], height=skw["height"], frames=skw["frames"], cst=cst, **ckw)


def checksum(stack):
    return int(stack.astype(np.int64).sum() + (stack.astype(np.int64) ** 2).sum() % 1000003)


def lag_fixture():
    out = {}
    for p, q, num in ((16, 8, 20000), (16, 6, 10000), (16, 7, 50000), (32, 8, 50000)):
        lag, samp, mtab = oracle.lag_tables(p, q, num)
        out[f"lag_{p}_{q}_{num}"] = lag
        out[f"samp_{p}_{q}_{num}"] = samp
        out[f"mtab_{p}_{q}_{num}"] = mtab
    return out


def main():
    oracle.build()
    np.savez_compressed(os.path.join(HERE, "lag_tables.npz"), **lag_fixture())
    for name in CASES:
        skw, cfg = case_config(name)
        stack = brownian_stack(**skw)
        r = oracle.run(stack, **oracle_kwargs(cfg))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), acf=r["acf"], var=r["var"],
                            blocked_ind=r["blocked_ind"], blocked_ok=r["blocked_ok"], fitres=r["fitres"],
                            chi2=r["chi2"], fitted=r["fitted"], stack_checksum=np.array([checksum(stack)]),
                            config=np.array(json.dumps(CASES[name])))
        print(name, "fitted", int(r["fitted"].sum()), "of", r["fitted"].size)


if __name__ == "__main__":
    main()
