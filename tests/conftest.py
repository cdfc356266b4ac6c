"""Shared test set-up: import paths, the `gpu` marker, and seeded marker sets.

Markers follow the reference's Julia layout (N x 2, column-major). Sizes mirror
the benchmark configurations: 16x16 mesh on [-6,6]^2 with N = 2048
(anisotropic Gaussian), 32x32 on [-8,8]^2 with N = 16384 (bimodal at +-2).
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "collisionoperators.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def gaussian_markers(N, sx=1.0, sy=0.5, seed=0, peak=0.0):
    """Anisotropic Gaussian (peak == 0) or balanced bimodal mixture at +-peak in v1
    (main.jl:91-103), uniform weights 1/N."""
    rng = np.random.default_rng(seed)
    v = np.zeros((N, 2), order="F")
    if peak != 0.0:
        half = N // 2
        centers = np.concatenate([np.full(half, -peak), np.full(N - half, peak)])
        v[:, 0] = centers + sx * rng.standard_normal(N)
    else:
        v[:, 0] = sx * rng.standard_normal(N)
    v[:, 1] = sy * rng.standard_normal(N)
    w = np.full(N, 1.0 / N)
    return v, w


def uniform_bp(lo, hi, n):
    return np.linspace(lo, hi, n + 1)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def collops_mod():
    import collops
    return collops


@pytest.fixture(scope="session")
def built_lib():
    """Build libcollops.so (nvcc cross-compiles without a GPU)."""
    import build as pkg_build
    return pkg_build.build()


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
