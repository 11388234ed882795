"""C ABI hygiene on the CPU: the library loads, exports every symbol that
include/*.h declares, struct layouts agree with the bindings, defaults equal
the reference defaults, and argument errors come back as status codes.
No call here launches GPU work."""
import ctypes as C
import re
from pathlib import Path

import pytest

from skyrendering_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(skyr_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = _abi.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_every_declared_symbol():
    assert set(declared_functions()) <= set(_abi.exported_symbols())


def test_struct_layouts_match():
    lib = _abi.lib()
    for sid, st in _abi.STRUCT_IDS.items():
        assert lib.skyr_struct_size(sid) == C.sizeof(st), st.__name__
    assert lib.skyr_struct_size(9999) == 0


def test_abi_version_and_status_strings():
    lib = _abi.lib()
    assert lib.skyr_abi_version() == 1
    assert lib.skyr_status_string(_abi.SKYR_EINVAL) == b"SKYR_EINVAL"
    assert lib.skyr_status_string(12345) == b"SKYR_UNKNOWN"


def test_defaults_are_reference_defaults():
    # AtmosphereParameters defaults (src/SkyRendering/Atmosphere.h:13-38)
    p = _abi.AtmosphereParameters()
    _abi.call("skyr_atmosphere_parameters_default", C.byref(p))
    assert p.bottom_radius == 6360.0 and p.thickness == pytest.approx(60.0)
    assert p.sun_angular_radius == pytest.approx(0.2667)
    assert list(p.rayleigh_scattering) == pytest.approx([0.175287, 0.409607, 1.0])
    assert p.rayleigh_scattering_scale == pytest.approx(0.0331)
    assert p.mie_phase_g == pytest.approx(0.8) and p.mie_absorption_scale == pytest.approx(0.000444)
    assert list(p.ozone_absorption) == pytest.approx([0.345561, 1.0, 0.045189])
    assert p.transmittance_steps == 40.0 and p.multiscattering_steps == 30.0 and p.multiscattering_mask == 1.0


def test_null_arguments_are_einval():
    lib = _abi.lib()
    s = _abi.LutSizes()
    p = _abi.AtmosphereParameters()
    assert lib.skyr_update_luts(None, C.byref(p), 1, C.byref(s), None, None) == _abi.SKYR_EINVAL
    assert b"null context" in lib.skyr_last_error()
    assert lib.skyr_ctx_create(None, None) == _abi.SKYR_EINVAL
    assert lib.skyr_ctx_destroy(None) == _abi.SKYR_OK


def test_lut_bytes():
    from skyrendering_gb300 import workloads as W

    s = W.plain_lut_sizes()
    lib = _abi.lib()
    assert lib.skyr_lut_bytes(C.byref(s), _abi.SKYR_LUT_TRANSMITTANCE) == 256 * 64 * 16
    assert lib.skyr_lut_bytes(C.byref(s), _abi.SKYR_LUT_SKY_VIEW) == 192 * 108 * 16
    s.format = _abi.SKYR_FORMAT_RGBA16F
    assert lib.skyr_lut_bytes(C.byref(s), _abi.SKYR_LUT_AERIAL_PERSPECTIVE) == 32 ** 3 * 8
    assert lib.skyr_lut_bytes(C.byref(s), _abi.SKYR_LUT_TRANSMITTANCE) == 256 * 64 * 16  # always FP32


def test_product_package_never_imports_the_oracle():
    pkg = ROOT / "skyrendering_gb300"
    for f in pkg.rglob("*.py"):
        assert "oracle" not in re.findall(r"^\s*(?:from|import)\s+(\w+)", f.read_text(), flags=re.M), f


def test_device_limits_defaults():
    d = _abi.DeviceLimits()
    _abi.call("skyr_device_limits_default", C.byref(d))
    assert d.tracking_steps == 1 << 20 and d.reserved == 0 and d.copy_wait_cycles == 1 << 31
    assert _abi.lib().skyr_ctx_set_limits(None, C.byref(d)) == _abi.SKYR_EINVAL


def _fields_equal(a, b):
    from skyrendering_gb300.config import struct_dict

    return struct_dict(a) == struct_dict(b)


def test_loader_defaults_equal_library_defaults():
    """The reference defaults the config loader restates (no CUDA library needed)
    are the library's skyr_*_default, field for field."""
    from skyrendering_gb300 import config as K

    p = _abi.AtmosphereParameters()
    _abi.call("skyr_atmosphere_parameters_default", C.byref(p))
    assert _fields_equal(K.atmosphere_defaults(), p)
    c = _abi.CloudParameters()
    _abi.call("skyr_cloud_parameters_default", C.byref(c))
    assert _fields_equal(K.cloud_defaults(), c)
    for kind in (_abi.SKYR_MATERIAL_DEFAULT0, _abi.SKYR_MATERIAL_DEFAULT1, _abi.SKYR_MATERIAL_MINIMAL,
                 _abi.SKYR_MATERIAL_VOXEL):
        m = _abi.CloudMaterial()
        _abi.call("skyr_cloud_material_default", kind, C.byref(m))
        assert _fields_equal(K.material_defaults(kind), m), kind
