"""Writes tests/golden/reference_configs.json: the skyr parameter blocks that
skyrendering_gb300.config.load() makes of the reference's four configuration
files (bin/config.json, config2.json, config3.json, config_voxel.json), as
plain field dicts.  The GPU test renders a frame from these blocks on a
machine without the reference; the CPU test re-parses the files (where they
are mounted) and checks that the loader still gives these values.

    python tests/golden/make_reference_configs.py [path/to/reference]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from skyrendering_gb300 import config as K  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_configs.json"
FILES = ("config.json", "config2.json", "config3.json", "config_voxel.json")


def blocks(cfg: K.ReferenceConfig) -> dict:
    return {"atmosphere": K.struct_dict(cfg.atmosphere), "render": K.struct_dict(cfg.render),
            "composite": K.struct_dict(cfg.composite), "cloud": K.struct_dict(cfg.cloud),
            "material": K.struct_dict(cfg.material), "lut_sizes": K.struct_dict(cfg.lut_sizes),
            "noise": {k: K.struct_dict(v) for k, v in cfg.noise.items()},
            "camera": {"position": list(cfg.camera.position), "front": list(cfg.camera.front),
                       "up": list(cfg.camera.up), "fovy": cfg.camera.fovy, "aspect": cfg.camera.aspect,
                       "z_near": cfg.camera.z_near, "z_far": cfg.camera.z_far},
            "init": cfg.init, "extra": cfg.extra}


def main(reference: str = "/root/reference") -> None:
    out = {f: blocks(K.load(Path(reference) / "bin" / f, strict=True)) for f in FILES}
    OUT.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{OUT}: {', '.join(out)}")


if __name__ == "__main__":
    main(*sys.argv[1:])
