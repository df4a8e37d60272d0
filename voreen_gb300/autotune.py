"""Autotuner for the march: ray-tile shape, brick size and empty-space cell
size, chosen by timing candidates on the device.

Requests are grouped by a class key (dtype, volume size class, image size
class); for each class the tuner renders one representative request with
every candidate, keeps the fastest (median kernel time of a few frames) and
caches it. Brick size is an upload-time choice, so tuning it re-uploads the
representative volume once per candidate brick size.
"""
from __future__ import annotations

import itertools
import json
import math
import os
import statistics

from . import EE_ANALYTIC, OUT_RGBA8, TransferFunction, Volume, render

TILE_WIDTHS = (4, 8, 16)
BRICKS = (16, 32)
SKIP_CELLS = (2, 4, 8, 16)


def class_key(dtype: int, dims, width: int, height: int) -> str:
    """Request class the tuned settings are cached under: dtype, log2 of the
    largest volume dimension, log4 of the pixel count (both rounded)."""
    vclass = int(round(math.log2(max(dims))))
    iclass = int(round(math.log2(max(1, width * height)) / 2))
    return f"dt{dtype}-v{vclass}-i{iclass}"


class Autotuner:
    """Times the candidate tile widths, brick sizes and skip cells on one
    representative request per class and keeps the fastest (optionally
    persisted as JSON at cache_path)."""

    def __init__(self, ctx, cache_path: str | None = None, frames: int = 3):
        self.ctx = ctx
        self.frames = frames
        self.cache_path = cache_path
        self.table: dict[str, dict] = {}
        # per class, every candidate timed in this session: (tile_width, brick, skip_cell, kernel_ms)
        self.timings: dict[str, list] = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                self.table = json.load(f)

    def save(self):
        if self.cache_path:
            with open(self.cache_path, "w") as f:
                json.dump(self.table, f, indent=1, sort_keys=True)

    def _time(self, vol, tf, params) -> float:
        ms = []
        for _ in range(self.frames + 1):
            _, st = render(self.ctx, vol, tf, params, None, None, OUT_RGBA8, self._out(params))
            ms.append(st.kernel_ms)
        return statistics.median(ms[1:])

    def _out(self, params):
        import torch
        key = (params.width, params.height)
        if getattr(self, "_buf_key", None) != key:
            self._buf = torch.empty((params.height, params.width, 4), dtype=torch.uint8, device="cuda")
            self._buf_key = key
        return self._buf

    def tune(self, voxels, spacing, tf_rgba, domain, params, tune_bricks: bool = True) -> dict:
        """Best {tile_width, brick, skip_cell, kernel_ms} for this request's class."""
        dims = (voxels.shape[2], voxels.shape[1], voxels.shape[0])
        key = class_key(_dtype_of(voxels), dims, params.width, params.height)
        if key in self.table:
            return self.table[key]
        best = None
        timed = self.timings.setdefault(key, [])
        bricks = BRICKS if tune_bricks else (32,)
        params.entry_exit_mode = EE_ANALYTIC
        for brick in bricks:
            vol = Volume(self.ctx, voxels, spacing, brick_size=brick)
            tf = TransferFunction(self.ctx, tf_rgba, domain)
            for tw, cell in itertools.product(TILE_WIDTHS, SKIP_CELLS):
                if cell > brick:
                    continue
                params.tile_width = tw
                params.skip_cell_size = cell
                ms = self._time(vol, tf, params)
                timed.append((tw, brick, cell, ms))
                if best is None or ms < best["kernel_ms"]:
                    best = {"tile_width": tw, "brick": brick, "skip_cell": cell, "kernel_ms": ms}
            tf.close()
            vol.close()
        self.table[key] = best
        return best


def _dtype_of(voxels) -> int:
    import numpy as np
    return {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.float32): 2}[voxels.dtype]
