"""Builds libimfcs_gb300.so in-tree for sm_103a (GB300) with nvcc.

Usage: python -m imaging_fcs_1_52_gb300.build  (or build() from Python).
The translation units compile in parallel; the result lands next to this
file so that the tests, the bench and the smoke check load the in-tree copy.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libimfcs_gb300.so")
SOURCES = ["imfcs_stream.cu", "imfcs_corr2.cu", "imfcs_prep.cu", "imfcs_corr.cu", "imfcs_fit.cu", "imfcs_lm3.cu", "imfcs_lm5.cu", "imfcs_lm11.cu", "imfcs_lm_tirf.cu", "imfcs_gls.cu", "imfcs_capi.cu",
           "imfcs_ref_api.cu", "imfcs_sim.cu", "imfcs_noalloc.cu", "imfcs_mlp.cu", "imfcs_batch.cu", "imfcs_ingest.cu",
           "imfcs_band.cu", "imfcs_probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> str:
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "imfcs_gb300.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
