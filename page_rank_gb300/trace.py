"""NVTX ranges around the engine's phases (builds, SpMMs, chunks of power
iteration steps, server rounds), so a timeline profiler shows them next to
the kernels.  Host-side markers only: nothing is captured into CUDA graphs,
and they cost a few microseconds per range.  ``GL_NVTX=0`` turns them off."""
from __future__ import annotations

import contextlib
import os

import torch

_ON = os.environ.get("GL_NVTX", "1") != "0"


@contextlib.contextmanager
def nvtx_range(name: str):
    if not (_ON and torch.cuda.is_available()):
        yield
        return
    torch.cuda.nvtx.range_push(name)
    try:
        yield
    finally:
        torch.cuda.nvtx.range_pop()
