"""Endless frozen-flow screen extruded row by row on the GB300
(drop-in for ``pyturb.InfinitePhaseScreen``, ``src/pyturb/infinite.py:120-395``).

The ``(cap, n)`` ring lives on the device; each new row is one native
extrusion call (``A z + B beta``), the pupil is one native row-interpolation
call. The host keeps the reference's ``base``/``fill`` compaction
bookkeeping (integers only) so clamping matches the reference exactly.
"""

from __future__ import annotations

from typing import Any, Union

import numpy as np

from . import _lib
from .backend import NoiseStream, dptr, stream_handle, torch_module
from .config import ScreenConfig
from .covariance import AnchorTables, anchor_modes, build_operator, phase_covariance
from .extrude import RingExtruder, compact_bounds
from .fourier import PhaseScreen

__all__ = ["InfinitePhaseScreen", "phase_covariance"]

_INTERP = {"linear": 0, "cubic": 1, "lanczos": 2}


class InfinitePhaseScreen:
    """Same constructor and methods as the reference (plus ``host_noise``)."""

    def __init__(self, n: int, pixel_scale: float, r0: float, L0: float = 25.0,
                 stencil_rows: int = 2, interp: str = "cubic", seed: Any = None,
                 device: str = "gpu", dtype: Union[str, np.dtype] = "float32",
                 host_noise=None) -> None:
        config = ScreenConfig.create(n, pixel_scale, r0, L0, device, dtype,
                                     finite_outer_scale=True)
        if (not isinstance(stencil_rows, (int, np.integer)) or isinstance(stencil_rows, bool)
                or not 1 <= stencil_rows < config.n):
            raise ValueError("stencil_rows must be in [1, n)")
        if interp not in ("cubic", "linear", "lanczos"):
            raise ValueError("interp must be 'cubic', 'linear', or 'lanczos'")
        self.n = config.n
        self.pixel_scale = config.pixel_scale
        self.r0 = config.r0
        self.L0 = config.L0
        self.stencil_rows = int(stencil_rows)
        self.interp = interp
        self.device = config.device
        self.dtype = config.dtype
        # FP64 device build at unit r0 (the reference's eigen-square-root B in
        # the parity mode, the build's Cholesky factor otherwise)
        op = build_operator(self.n, self.stencil_rows, self.pixel_scale, self.L0,
                            b_factor="eigh" if host_noise is not None else "cholesky",
                            want_float64=True)
        self._stream = NoiseStream(seed, host_noise)
        self._margin = self.stencil_rows + 6
        self._capacity = self.n + self._margin
        self._ring = RingExtruder(self.n, self.stencil_rows, self._capacity, [], [0],
                                  [self.r0 ** (-5.0 / 6.0)], [self._stream],
                                  device_operator=op.M,
                                  anchor=(AnchorTables([op], anchor_modes(self.n, ()))
                                          if anchor_modes(self.n, ()) else None))
        op.M64 = None
        gen = PhaseScreen(n=self.n, pixel_scale=self.pixel_scale, r0=self.r0, L0=self.L0,
                          _stream=self._stream, host_noise=host_noise)
        self._ring.seed_rows(0, gen.generate())
        del gen
        self._base = 0
        self._fill = self.n
        self._travel = 0.0
        self._current = None
        self._advance_to(0.0)

    def _advance_to(self, travel: float) -> None:
        if travel < self._travel:
            raise ValueError("wind travel is monotonic; travel cannot decrease")
        self._travel = float(travel)
        top = int(np.floor(self._travel)) + self.n + 2
        count = 0
        while self._base + self._fill - 1 < top:
            if self._fill == self._capacity:
                self._base, self._fill = compact_bounds(self._base, self._fill,
                                                        self.stencil_rows, self._travel)
            self._fill += 1
            count += 1
        self._ring.extrude([count])
        torch = torch_module()
        out = torch.empty((self.n, self.n), dtype=torch.float32, device=self._ring.buf.device)
        _lib.call("pt_rows_sample", self.n, self._capacity, _INTERP[self.interp],
                  self._base % self._capacity, self._fill - 1, self._travel - self._base,
                  dptr(self._ring.buf), dptr(out), stream_handle())
        self._current = out

    @property
    def screen(self):
        return self._current

    def step(self, steps: int = 1):
        steps = int(steps)
        if steps < 1:
            raise ValueError("steps must be >= 1")
        self._advance_to(self._travel + steps)
        return self._current

    def advance(self, pixels: float):
        pixels = float(pixels)
        if pixels < 0:
            raise ValueError("pixels must be >= 0 (wind travel is monotonic)")
        self._advance_to(self._travel + pixels)
        return self._current

    @property
    def travel(self) -> float:
        return self._travel

    def __repr__(self) -> str:
        return (f"InfinitePhaseScreen(n={self.n}, pixel_scale={self.pixel_scale}, "
                f"r0={self.r0}, L0={self.L0}, stencil_rows={self.stencil_rows}, "
                f"interp={self.interp!r}, device={self.device!r}, dtype={self.dtype.name!r})")
