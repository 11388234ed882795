"""Committed fixtures and the scripts that made them."""
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def reference_blue_noise() -> np.ndarray:
    """The reference's 64x64 blue-noise jitter tile (data/BlueNoise/64_64/HDR_L_0.png)
    as the float32 values its GL_R16 texture returns (value / 65535)."""
    return (np.load(HERE / "blue_noise_64x64.npy").astype(np.float64) / 65535.0).astype(np.float32)
