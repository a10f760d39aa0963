"""Builds libsphgpu.so in-tree with nvcc for sm_103a (make -C csrc)."""
from __future__ import annotations

import os
import shutil
import subprocess

from ._lib import LIB_PATH, PKG_ROOT

CSRC = os.path.join(PKG_ROOT, "csrc")


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build_library(jobs: int = 8, verbose: bool = False) -> str:
    """Compiles csrc/*.cu into libsphgpu.so (incremental; returns its path)."""
    cmd = ["make", "-C", CSRC, f"-j{jobs}", f"NVCC={nvcc_path()}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building libsphgpu.so failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stdout)
    return LIB_PATH
