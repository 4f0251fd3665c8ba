"""Helpers shared by the GPU tests."""
import numpy as np
import pytest


def engine_or_skip():
    """The engine module; GPU tests need a built library and a GPU (no fallback)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import mps_gb300
    from mps_gb300 import engine

    engine.load(build_if_missing=True)
    return mps_gb300


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)
