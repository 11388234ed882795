"""Host-side mirror of VolumetricCloud::PathTracing over the C ABI
(src/SkyRendering/VolumetricCloud.h:90-136, .cpp:495-581): a dense FP16 density
grid with its brick majorants, progressive accumulation and the display pass.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _abi
from .atmosphere import Context, LutSet, _ptr


class DensityGrid:
    """Dense half-precision grid placed in the local cloud frame (km)."""

    def __init__(self, nx: int, ny: int, nz: int, origin, voxel_size: float, density: float, brick: int = 16,
                 device="cuda"):
        self.data = torch.empty((nz, ny, nx), dtype=torch.float16, device=device)
        lib = _abi.lib()
        bx, by, bz = (lib.skyr_grid_brick_count(n, brick) for n in (nx, ny, nz))
        self.majorant = torch.zeros((bz, by, bx), dtype=torch.float32, device=device)
        self.struct = _abi.DensityGrid()
        g = self.struct
        g.data = self.data.data_ptr()
        g.nx, g.ny, g.nz = nx, ny, nz
        g.origin[:] = list(origin)
        g.voxel_size = voxel_size
        g.density = density
        g.majorant = self.majorant.data_ptr()
        g.brick = brick

    def generate(self, ctx: Context, gen: _abi.GridGenerator) -> "DensityGrid":
        _abi.call("skyr_grid_generate", ctx.handle, C.byref(gen), _ptr(self.data))
        return self.update_majorants(ctx)

    def update_majorants(self, ctx: Context) -> "DensityGrid":
        _abi.call("skyr_grid_majorants", ctx.handle, C.byref(self.struct), _ptr(self.majorant))
        return self

    def normalize_extinction(self, ctx: Context, sigma_max: float) -> "DensityGrid":
        """Set `density` so that the grid's largest voxel has extinction
        `sigma_max` (the global max comes from a density-1 majorant pass)."""
        self.struct.density = 1.0
        self.update_majorants(ctx)
        ctx.synchronize()
        m = float(self.majorant.max().item())
        self.struct.density = sigma_max / m if m > 0 else 0.0
        return self.update_majorants(ctx)


class PathTracer:
    """PathTracing: accumulates frames of one view."""

    def __init__(self, ctx: Context, params: _abi.PathtraceParameters, cloud: _abi.CloudParameters,
                 view: _abi.CloudView, env_view: _abi.AtmosphereRenderParameters, sizes: _abi.LutSizes,
                 grid: DensityGrid | None = None, material: _abi.CloudMaterial | None = None,
                 textures: _abi.CloudTextures | None = None, track_variance: bool = False):
        self.ctx, self.params, self.cloud, self.view, self.env_view, self.sizes = ctx, params, cloud, view, env_view, sizes
        self.grid, self.material, self.textures = grid, material, textures
        self.acc = torch.zeros((view.height, view.width, 4), dtype=torch.float32, device="cuda")
        self.acc_sq = torch.zeros_like(self.acc) if track_variance else None
        self.frames = 0

    def reset(self):
        self.acc.zero_()
        if self.acc_sq is not None:
            self.acc_sq.zero_()
        self.frames = 0

    def render(self, atmosphere: _abi.AtmosphereParameters, luts: LutSet, n_frames: int = 1, region=None):
        reg = None if region is None else (C.c_int * 4)(*region)
        _abi.call("skyr_pathtrace", self.ctx.handle, C.byref(atmosphere), C.byref(self.cloud),
                  None if self.material is None else C.byref(self.material),
                  None if self.textures is None else C.byref(self.textures),
                  None if self.grid is None else C.byref(self.grid.struct), C.byref(self.params),
                  C.byref(self.view), C.byref(self.env_view), C.byref(self.sizes), _ptr(luts.transmittance),
                  _ptr(luts.sky_view_luminance), _ptr(luts.sky_view_transmittance),
                  _ptr(luts.aerial_perspective_luminance), _ptr(luts.aerial_perspective_transmittance),
                  self.frames + 1, n_frames, reg, _ptr(self.acc), _ptr(self.acc_sq))
        self.frames += n_frames
        return self

    def resolve(self, background: torch.Tensor | None = None) -> torch.Tensor:
        out = torch.empty((self.view.height, self.view.width, 4), dtype=torch.float16, device="cuda")
        _abi.call("skyr_pathtrace_resolve", self.ctx.handle, _ptr(self.acc), self.view.width, self.view.height,
                  max(self.frames, 1), _ptr(background), _ptr(out))
        return out
