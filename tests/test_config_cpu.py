"""The loader of the reference's configuration files (skyrendering_gb300.config),
on the CPU.

* Where the reference is mounted, its four files (bin/config.json,
  config2.json, config3.json, config_voxel.json) load in strict mode (no
  unknown key), a sample of fields equals the raw JSON, the camera's
  view-projection is glm's perspective x lookAt of the serialised vectors, and
  the blocks equal the committed fixture (tests/golden/reference_configs.json).
* Synthetic documents: absent members keep the reference defaults, dotted
  keys and the material "type" dispatch, unknown keys (listed, or an error in
  strict mode), bad types and unknown materials give ConfigError.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from skyrendering_gb300 import _abi
from skyrendering_gb300 import config as K

REF = Path("/root/reference/bin")
GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_configs.json"
FILES = ("config.json", "config2.json", "config3.json", "config_voxel.json")
needs_reference = pytest.mark.skipif(not REF.exists(), reason="the reference's bin/ is not mounted")


@needs_reference
@pytest.mark.parametrize("name", FILES)
def test_reference_files_load_and_match_fixture(name):
    raw = json.loads((REF / name).read_text())
    cfg = K.load(REF / name, strict=True)
    assert cfg.unknown == []
    p = raw["earth_"]["parameters"]
    assert cfg.atmosphere.bottom_radius == pytest.approx(p["bottom_radius"])
    assert cfg.atmosphere.thickness == pytest.approx(p["thickness"])
    assert list(cfg.atmosphere.rayleigh_scattering) == pytest.approx(p["rayleigh_scattering"])
    assert cfg.atmosphere.mie_absorption_scale == pytest.approx(p["mie_absorption_scale"])
    r = raw["atmosphere_render_parameters_"]
    assert cfg.render.sun_direction_theta == pytest.approx(r["sun_direction_theta"])
    assert cfg.render.aerial_perspective_lut_max_distance == pytest.approx(r["aerial_perspective_lut_max_distance"])
    assert cfg.composite.raymarching_steps == pytest.approx(r["raymarching_steps"])
    assert cfg.lut_sizes.aerial_perspective_depth == raw["atmosphere_render_init_parameters_"][
        "aerial_perspective_lut_depth"]
    vc = raw["volumetric_cloud_"]
    assert cfg.cloud.bottom_altitude == pytest.approx(vc["bottom_altitude_"])
    assert cfg.cloud.max_raymarch_steps == pytest.approx(vc["max_raymarch_steps_"])
    assert list(cfg.cloud.env_color) == pytest.approx(vc["env_color_"])
    m = vc["material"]
    assert cfg.material.type == K.MATERIAL_TYPES[m["type"]]
    data = m["data"]
    if "materail_common_" in data:
        com = data["materail_common_"]
        assert cfg.material.density == pytest.approx(com["density_"])
        assert cfg.material.cloud_map_repeat_size == pytest.approx(com["cloud_map_.texture.repeat_size"])
        cm = cfg.noise["cloud_map"]
        assert cm.channel[0].a.base_frequency == com["cloud_map_.buffer.uDensity.base_frequency"]
        assert cm.channel[1].a.remap_min == pytest.approx(com["cloud_map_.buffer.uHeight.remap_min"])
        assert cfg.noise["detail"].channel[0].b.base_frequency == com["detail_.buffer.uWorley.base_frequency"]
        assert cfg.material.minfilter3d == K.MIPMAP_MIN[com["minfilter3d_"]]
    else:
        assert cfg.material.density == pytest.approx(data["density_"])
        assert list(cfg.material.voxel_width) == pytest.approx(data["width_"])
    # ProjectionMatrix() * ViewMatrix() of the serialised vectors (Camera.cpp:13-19)
    cam = raw["camera_"]
    eye, f, up = (np.array(cam[k], dtype=np.float64) for k in ("position_", "front_", "up_"))
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = [-s @ eye, -u @ eye, f @ eye]
    t = np.tan(np.radians(cam["fovy"]) / 2)
    n, fa = cam["zNear"], cam["zFar"]
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = 1 / (cam["aspect_"] * t), 1 / t
    proj[2, 2], proj[2, 3], proj[3, 2] = -(fa + n) / (fa - n), -2 * fa * n / (fa - n), -1
    want = (proj @ view).flatten(order="F")
    assert np.allclose(np.array(cfg.render.view_projection), want, rtol=1e-5, atol=1e-6)
    # the committed fixture is what the loader makes of the file
    fixture = json.loads(GOLDEN.read_text())[name]
    from tests.golden.make_reference_configs import blocks

    assert json.loads(json.dumps(blocks(cfg), sort_keys=True)) == fixture


def test_fixture_round_trips_to_structs():
    fixture = json.loads(GOLDEN.read_text())
    for name in FILES:
        cfg = K.from_blocks(fixture[name])
        assert K.struct_dict(cfg.atmosphere) == fixture[name]["atmosphere"]
        assert K.struct_dict(cfg.noise["detail"]) == fixture[name]["noise"]["detail"]
        v = cfg.view(320, 180)
        assert v.width == 320 and v.viewport_height == 180
        assert v.sun_direction_theta == cfg.render.sun_direction_theta


def test_absent_members_keep_reference_defaults():
    cfg = K.load({})
    assert K.struct_dict(cfg.atmosphere) == K.struct_dict(K.atmosphere_defaults())
    assert K.struct_dict(cfg.cloud) == K.struct_dict(K.cloud_defaults())
    assert cfg.material.type == _abi.SKYR_MATERIAL_DEFAULT0  # VolumetricCloud's default material
    assert cfg.render.sun_direction_theta == 70.0 and cfg.lut_sizes.aerial_perspective_depth == 32
    assert cfg.noise["cloud_map"].octaves == 8 and cfg.noise["detail"].width == 128


def test_dotted_keys_and_material_dispatch():
    doc = {"volumetric_cloud_": {"thickness_": 3.0, "material": {
        "type": "class VolumetricCloudDefaultMaterial1",
        "data": {"edge_cut_": 0.5, "materail_common_": {"detail_.buffer.uPerlin.seed": 9,
                                                          "detail_.texture.repeat_size": 7.5,
                                                          "minfilter2d_": "LINEAR_MIPMAP_LINEAR",
                                                          "wind_speed_": 0.25}}}}}
    cfg = K.load(doc, strict=True)
    assert cfg.cloud.thickness == 3.0
    assert cfg.material.type == _abi.SKYR_MATERIAL_DEFAULT1 and cfg.material.edge_cut == pytest.approx(0.5)
    assert cfg.noise["detail"].channel[0].a.seed == 9
    assert cfg.material.detail_repeat_size == pytest.approx(7.5)
    assert cfg.material.minfilter2d == _abi.SKYR_MIPMAP_LINEAR_MIPMAP_LINEAR
    assert cfg.extra["wind_speed"] == pytest.approx(0.25)
    mini = K.load({"volumetric_cloud_": {"material": {"type": "class VolumetricCloudMinimalMaterial",
                                                      "data": {"density_": 2.0}}}})
    assert mini.material.type == _abi.SKYR_MATERIAL_MINIMAL and mini.material.density == 2.0


def test_unknown_keys_are_reported_not_fatal():
    doc = {"no_such_member": 1, "earth_": {"parameters": {"thickness": 80.0, "bogus": 2}}}
    cfg = K.load(doc)
    assert sorted(cfg.unknown) == ["earth_.parameters.bogus", "no_such_member"]
    assert cfg.atmosphere.thickness == 80.0
    with pytest.raises(K.ConfigError, match="unknown key"):
        K.load(doc, strict=True)


@pytest.mark.parametrize("doc", [
    {"volumetric_cloud_": {"material": {"type": "class NoSuchMaterial", "data": {}}}},
    {"earth_": {"parameters": {"thickness": "thick"}}},
    {"earth_": {"parameters": {"ground_albedo": [0.1, 0.2]}}},
    {"atmosphere_render_init_parameters_": {"aerial_perspective_lut_depth": 1.5}},
    {"volumetric_cloud_": {"material": {"type": "class VolumetricCloudDefaultMaterial1", "data": {
        "materail_common_": {"minfilter3d_": "CUBIC"}}}}},
    {"camera_": {"front_": [0, 0, 0], "up_": [0, 1, 0]}},
    "[1, 2]",
])
def test_bad_documents_raise_config_error(doc):
    with pytest.raises(K.ConfigError):
        K.load(doc)
