"""Shared fixtures of the test suite: seeded models, cameras, GPU checks."""
from __future__ import annotations

import functools
import os

import numpy as np
import pytest

from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@functools.lru_cache(maxsize=None)
def tiny_model(seed: int = 7, nlvl: int = 1) -> str:
    return fmodel.ensure_model(fmodel.spec_tiny(seed=seed, nlvl=nlvl))


def small_camera(seed: int, W: int, H: int, radius: float = 4.0) -> dict:
    return fcam.seeded_camera(seed, radius=radius, width=W, height=H)


def psnr(a, b, peak=1.0):
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)
