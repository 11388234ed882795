"""A frame rendered from the reference's own configuration files, on the GPU.

The parameter blocks are what skyrendering_gb300.config.load() makes of
bin/config.json (Material1) and bin/config2.json (Material0) -- committed as
tests/golden/reference_configs.json, since the reference is not present where
the GPU tests run.  Everything comes from the file: the atmosphere, the LUT
sizes (sky-view 128x128, aerial perspective 32x32xdepth over the configured
distance), the cloud layer and lighting, the material and its three generated
noise textures (512^2 RG8, 128^3 R8 Perlin-Worley, 128^2 RGBA8 displacement,
8 fBm octaves), the camera and sun; the jitter is the reference's own
blue-noise tile.  Checked against the FP64 oracle on the same textures and
LUTs: <= 1e-3 mean relative error per output, as the other frame tests.
"""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import config as K
from skyrendering_gb300.atmosphere import update_lut_set
from skyrendering_gb300.cloud import NoiseTexture, VolumetricCloud, prepare_textures, textures_struct
from tests.golden import reference_blue_noise

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_configs.json"
MEAN_TOL = 1e-3


def mean_rel(got, want):
    return float(np.abs(got - want).sum() / max(np.abs(want).sum(), 1e-300))


@pytest.mark.parametrize("name", ["config.json", "config2.json"])
def test_frame_from_reference_config(ctx, name):
    cfg = K.from_blocks(json.loads(GOLDEN.read_text())[name])
    w, h = 480, 270
    render = cfg.render_parameters(w, h)
    luts = update_lut_set(ctx, cfg.atmosphere, render, cfg.lut_sizes)
    tex = {k: NoiseTexture(d).generate(ctx) for k, d in cfg.noise.items()}
    prepare_textures(ctx, cfg.material.type, tex)
    bn = torch.from_numpy(reference_blue_noise()).cuda()
    view = cfg.view(w, h)
    vc = VolumetricCloud(ctx, cfg.cloud, cfg.material, textures_struct(**tex))
    rgba, dist = vc.render(cfg.atmosphere, view, cfg.lut_sizes, luts, bn)
    ctx.synchronize()
    ctx.check_status()
    host = {k: (t.desc, t.data.cpu().numpy()) for k, t in tex.items()}
    o_rgba, o_dist = orc.cloud_render(cfg.atmosphere, cfg.cloud, cfg.material, host, view, cfg.lut_sizes,
                                      luts.transmittance[0].cpu().double().numpy(),
                                      luts.aerial_perspective_luminance[0].float().cpu().double().numpy(),
                                      luts.aerial_perspective_transmittance[0].float().cpu().double().numpy(),
                                      bn.cpu().numpy())
    g = rgba.float().cpu().numpy().reshape(-1, 4).astype(np.float64)
    gd = dist.cpu().numpy().reshape(-1).astype(np.float64)
    err = {"luminance": mean_rel(g[:, :3], o_rgba[:, :3]), "transmittance": mean_rel(g[:, 3], o_rgba[:, 3]),
           "distance": mean_rel(gd, o_dist)}
    print(f"{name}: " + ", ".join(f"{k}={v:.2e}" for k, v in err.items()) +
          f"; cloud cover {(g[:, 3] < 0.999).mean():.2f}")
    assert all(v <= MEAN_TOL for v in err.values()), err
    assert np.isfinite(g).all()
    assert (g[:, 3] < 0.999).mean() > 0.01, "the configured view should contain cloud"
    # the LUT set of the configured atmosphere against the oracle (<= 1e-3 per texel)
    ref = orc.lut_set(cfg.atmosphere, render, cfg.lut_sizes, 64)
    for n in ("transmittance", "multiscattering", "sky_view_luminance", "aerial_perspective_luminance"):
        got = getattr(luts, n)[0].float().cpu().numpy().astype(np.float64)[..., :3]
        want = ref[n][..., :3]
        assert (np.abs(got - want) / np.maximum(np.abs(want), 1e-300)).max() <= 1e-3, n
