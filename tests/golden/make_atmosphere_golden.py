"""Generate tests/golden/atmosphere_small.npz from the FP64 CPU oracle.

The reference ships no golden vectors (it has no tests), so these fixtures are
the oracle's own outputs on a reduced-size Earth-like configuration; they pin
the oracle against regressions and give the GPU tests a fixed target.
Run:  python tests/golden/make_atmosphere_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402
from skyrendering_gb300 import workloads as W  # noqa: E402


def small_sizes():
    s = W.plain_lut_sizes()
    s.transmittance_width, s.transmittance_height = 32, 16
    s.multiscattering_width, s.multiscattering_height = 8, 8
    s.sky_view_width, s.sky_view_height = 24, 16
    s.aerial_perspective_width = s.aerial_perspective_height = s.aerial_perspective_depth = 8
    return s


def cases():
    p = W.earth_like_atmosphere()
    cam = W.frame_camera()
    for z in W.SUN_ZENITHS_DEG:
        yield f"z{int(z)}", p, W.render_parameters(cam, z)


def main():
    s = small_sizes()
    out = {}
    for tag, p, r in cases():
        o = orc.lut_set(p, r, s, 64)
        for k, v in o.items():
            out[f"{tag}/{k}"] = v
    np.savez_compressed(Path(__file__).with_name("atmosphere_small.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
