"""Non-periodic frozen flow by Assemat-Wilson row extrusion on the GB300
(drop-in for ``pyturb.extrude.ExtrudedAtmosphere``).

Setup (device, FP64, once per outer scale): the operator ``M = [A | B_unit]``
(W x K float32, K = (m+1) W plus any sparse stencil points) from one
factorisation of the joint stencil/new-row covariance (``covariance.py``;
the reference builds it on the host, ``src/pyturb/extrude.py:250-304``).

Device state: one ``(L, cap, W)`` float32 slab of ring buffers. Virtual row v
of a layer sits in physical row ``(v - v0) mod cap``, so the wind advances an
index. The host keeps the reference's ``base``/``fill`` bookkeeping,
compaction included (``src/pyturb/ring.py:9-28``), purely as integers: it
fixes which rows a readout may touch (its clamp range) exactly as the
reference does, without moving any data.

Per frame: all layers' new rows for one row step are one native GEMM
(``pt_extrude_rows``), then one fused readout kernel samples every layer's
rotated, magnified, shifted pupil grid and sums the layers
(``pt_readout``, the reference's ``extrude_readout_*`` kernels).
"""

from __future__ import annotations

import ctypes as C
from math import floor
from typing import Any, List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _lib
from .backend import NoiseStream, cuda_device, dptr, stream_handle, torch_module, upload
from .config import ExtrusionConfig
from .covariance import (AnchorTables, anchor_modes, build_extrusion, build_operator,
                         phase_covariance, sparse_points)
from .fourier import PhaseScreen

__all__ = ["ExtrudedAtmosphere", "build_extrusion", "phase_covariance", "RingExtruder"]

_INTERP = {"linear": 0, "cubic": 1, "lanczos": 2}


def _smooth_size(n: int) -> int:
    """Smallest 2^a 3^b >= n (a fast transform size for the seed screen)."""
    best = 1 << max(0, int(n - 1).bit_length())
    p3 = 1
    while p3 < 2 * n:
        v = p3
        while v < n:
            v *= 2
        best = min(best, v)
        p3 *= 3
    return best


class _RowQueue:
    """A noise stream that hands out pre-drawn rows (the boil stream's draws,
    taken in the reference's order and replayed to a scratch extrusion)."""

    key = 0

    def __init__(self, injected: bool) -> None:
        self.injected = injected
        self.rows: list = []

    def draw(self, shape):
        return self.rows.pop(0)


def along_extent_and_span(n: int, vx: float, vy: float, mag: float,
                          fov_margin_pix: float) -> Tuple[float, int]:
    """A layer's along-wind half extent and buffer span (``src/pyturb/extrude.py:222-247``)."""
    speed = float(np.hypot(vx, vy))
    c = vx / speed if speed > 0 else 1.0
    s = vy / speed if speed > 0 else 0.0
    half = (n - 1) / 2.0 * float(mag)
    ext = half * (abs(c) + abs(s))
    span = int(np.ceil(ext + fov_margin_pix)) - int(np.floor(-ext - fov_margin_pix)) + 3
    return ext, span


def compact_bounds(base: int, fill: int, depth: int,
                   first_readable_row: float) -> Tuple[int, int]:
    """New ``(base, fill)`` after the reference's ring compaction
    (``src/pyturb/ring.py:9-28``): rows below the readable window and the
    stencil (the last ``depth`` rows: the m full rows, or as deep as the
    sparse points reach) are dropped, at least one."""
    target = int(floor(first_readable_row)) - 1
    stencil = base + fill - depth
    keep_from = max(1, min(target, stencil) - base)
    return base + keep_from, fill - keep_from


class RingExtruder:
    """The device ring slabs plus the per-screen host bookkeeping.

    ``screens`` independent ring buffers of ``cap`` rows x ``W`` columns; screen
    s uses operator group ``groups[s]`` scaled by ``bscale[s]``. ``sparse``
    lists the stencil's sparse points ``(depth, column)`` after its ``m`` full
    rows (none: the reference's rows-only stencil). ``operators`` holds host
    ``(A, B)`` pairs, or ``device_operator`` an existing ``(G, W, K)``
    float32 CUDA tensor, K = (m + 1) W + len(sparse). ``operator_lo``
    (``(G, W, Kz)`` float32, ``A - float32(A)``) makes the FP32 form add that
    correction each step, so that the recursion follows the float64
    operator instead of accumulating the float32 rounding of ``A``.
    ``anchor`` (``AnchorTables``) makes the FP32 form recompute the 32
    smoothest modes of every new row in double-float arithmetic: the row
    recursion amplifies float32 rounding in those modes over long runs.
    ``increments``: the operator is in increment form (``build_operator(...,
    increments=True)``), the operand holds row differences and each new row
    is the newest stencil row plus the product."""

    FORMS = {"fp32": 0, "bf16x2": 2, "bf16x3": 3}

    def __init__(self, W: int, m: int, cap: int, operators: List[Tuple[np.ndarray, np.ndarray]],
                 groups: Sequence[int], bscale: Sequence[float], streams: Sequence[NoiseStream],
                 device_operator=None, form: str = "fp32",
                 sparse: Sequence[Tuple[int, int]] = (), operator_lo=None, anchor=None,
                 increments: bool = False):
        torch = torch_module()
        if form not in self.FORMS:
            raise ValueError(f"form must be one of {sorted(self.FORMS)}, got {form!r}")
        self.form = form
        self.terms = self.FORMS[form]
        self.W, self.m, self.cap = int(W), int(m), int(cap)
        self.sparse = [(int(d), int(c)) for d, c in sparse]
        self.ns = len(self.sparse)
        self._stencil = _lib.sparse_stencil(self.sparse)
        self._sp = C.byref(self._stencil) if self._stencil is not None else None
        self.depth = max([self.m] + [d for d, _ in self.sparse])
        if self.depth >= self.cap:
            raise ValueError("the ring must hold more rows than the stencil reaches back")
        self.S = len(groups)
        self.groups = [int(g) for g in groups]
        self.bscale = [float(b) for b in bscale]
        self.streams = list(streams)
        if device_operator is not None:
            self.M = device_operator if device_operator.dim() == 3 else device_operator[None]
        else:
            M = np.stack([np.concatenate([a, b], axis=1) for a, b in operators])
            self.M = upload(M)
        if self.M.shape[1:] != (self.W, (self.m + 1) * self.W + self.ns):
            raise ValueError(f"operator shape {tuple(self.M.shape)} does not match W={self.W}, "
                             f"m={self.m} and {self.ns} sparse points")
        self.G = int(self.M.shape[0])
        self.increments = bool(increments)
        self.anchor = anchor if self.terms == 0 else None
        self._anchor = C.byref(anchor.struct) if self.anchor is not None else None
        self.M_lo = None
        self.lo_tiles = None
        if operator_lo is not None and self.terms == 0:
            self.M_lo = operator_lo if operator_lo.dim() == 3 else operator_lo[None]
            if self.M_lo.shape != (self.G, self.W, self.m * self.W + self.ns):
                raise ValueError("operator_lo must be (G, W, m W + sparse points)")
            nbytes = int(_lib.load().pt_extrude_lo_bytes(self.W, self.m, self.ns, self.G))
            self.lo_tiles = torch.empty(nbytes, dtype=torch.uint8, device=cuda_device())
            _lib.call("pt_extrude_lo_prepare", self.W, self.m, self.ns, self.G,
                      dptr(self.M_lo.contiguous()), dptr(self.lo_tiles), nbytes, stream_handle())
        self.buf = torch.empty((self.S, self.cap, self.W), dtype=torch.float32,
                               device=cuda_device())
        # rows extruded so far per screen (relative virtual rows [0, top))
        self.top = np.zeros(self.S, dtype=np.int64)
        self._group = np.asarray(self.groups, dtype=np.int32)
        self._bscale = np.asarray(self.bscale, dtype=np.float32)
        self._key = np.asarray([st.key for st in self.streams], dtype=np.uint64)
        self.work_bytes = 0
        self.work = None
        self.tiles = None
        if self.terms:
            # the operator split into bf16 terms, tiled for the tensor cores (once)
            nbytes = int(_lib.load().pt_extrude_tc_operator_bytes(self.W, self.m, self.ns,
                                                                  self.G, self.terms))
            self.tiles = torch.empty(nbytes, dtype=torch.uint8, device=cuda_device())
            _lib.call("pt_extrude_tc_prepare", self.W, self.m, self.ns, self.G, dptr(self.M),
                      self.terms, dptr(self.tiles), nbytes, stream_handle())

    def _ensure_work(self, jobs_per_step: int) -> None:
        lib = _lib.load()
        if self.terms:
            need = int(lib.pt_extrude_tc_workspace_bytes(self.W, self.m, self.ns,
                                                         max(1, jobs_per_step), self.terms))
        else:
            need = int(lib.pt_extrude_workspace_bytes(self.W, self.m, self.ns,
                                                      max(1, jobs_per_step)))
        if need > self.work_bytes:
            torch = torch_module()
            self.work = torch.empty(need, dtype=torch.uint8, device=cuda_device())
            self.work_bytes = need

    def seed_rows(self, s: int, rows) -> None:
        """Copy the initial (span, W) rows of screen s into ring rows [0, span)."""
        k = rows.shape[0]
        self.buf[s, :k].copy_(rows)
        self.top[s] = k

    def extrude(self, counts: Sequence[int]) -> None:
        """Extrude ``counts[s]`` new rows on every screen s (one native call:
        as many row steps as the largest count, all screens of a step batched)."""
        counts = np.ascontiguousarray(counts, dtype=np.int32).reshape(self.S)
        steps = int(counts.max()) if counts.size else 0
        if steps <= 0:
            return
        noise = None
        if any(st.injected for st in self.streams):
            rows = [self.streams[s].draw((self.W,))
                    for k in range(steps) for s in range(self.S) if k < counts[s]]
            noise = upload(np.stack(rows))
        self._ensure_work(int((counts > 0).sum()))
        ptr = lambda a: a.ctypes.data  # noqa: E731
        if self.terms:
            _lib.call("pt_extrude_batch_tc", self.W, self.m, self._sp, int(self.increments),
                      self.cap, self.G,
                      dptr(self.tiles), self.terms, dptr(self.buf), self.S, ptr(self._group),
                      ptr(self._bscale), ptr(self._key), ptr(self.top), ptr(counts), dptr(noise),
                      dptr(self.work), self.work_bytes, stream_handle())
        else:
            _lib.call("pt_extrude_batch", self.W, self.m, self._sp, int(self.increments),
                      self.cap, self.G,
                      dptr(self.M), dptr(self.lo_tiles), self._anchor, dptr(self.buf), self.S,
                      ptr(self._group), ptr(self._bscale),
                      ptr(self._key), ptr(self.top), ptr(counts), dptr(noise), dptr(self.work),
                      self.work_bytes, stream_handle())


class _LayerGeom:
    """Per-layer geometry and reference bookkeeping (``src/pyturb/extrude.py:307-496``)."""

    def __init__(self, n, W, dx, vx, vy, altitude_los, m, mag, fov_margin_pix, history=0):
        speed = float(np.hypot(vx, vy))
        self.speed = speed
        self.cos = vx / speed if speed > 0 else 1.0
        self.sin = vy / speed if speed > 0 else 0.0
        self.altitude_pix = float(altitude_los) / dx
        self.mag = float(mag)
        g = (np.arange(n, dtype=np.float64) - (n - 1) / 2.0) * self.mag
        along = g[:, None] * self.cos + g[None, :] * self.sin
        self.along_min = float(along.min())
        self.along_max = float(along.max())
        self.fov = float(fov_margin_pix)
        extent_min = self.along_min - self.fov
        self.span = int(np.ceil(self.along_max + self.fov)) - int(np.floor(extent_min)) + 3
        # `history` older rows sit below the readable window for a sparse
        # stencil's deepest points (none for the rows-only stencil)
        self.history = int(history)
        self.base = int(np.floor(extent_min)) - 2 - self.history  # virtual row of buffer row 0
        self.v0 = self.base                         # virtual row of ring row 0
        self.fill = self.span + self.history
        self.travel = 0.0
        self.m = m

    def offsets_for_direction(self, thx: float, thy: float) -> Tuple[float, float]:
        dxp = self.altitude_pix * thx
        dyp = self.altitude_pix * thy
        return dxp * self.cos + dyp * self.sin, -dxp * self.sin + dyp * self.cos


class ExtrudedAtmosphere:
    """Multi-layer extrusion engine (``src/pyturb/extrude.py:499-915``).

    Constructor as the reference's plus
    - ``host_noise`` (parity mode: the reference's draw order, and the
      reference's eigen-square-root ``B``);
    - ``extrude_form``: ``"fp32"`` (FP32 SIMT products, the default),
      ``"bf16x2"`` or ``"bf16x3"`` (operands split into 2 or 3 bf16 terms and
      multiplied on the tensor cores with an fp32 accumulator);
    - ``stencil_columns`` (default 0): sparse stencil columns beside the
      ``stencil_rows`` full rows, each sampled at depths 4, 8, 16, ... up to
      ``sparse_depth`` rows back (default: the largest power of two not above
      the buffer width). ``stencil_rows=2, stencil_columns=2`` is the
      "2 full rows + 2 sparse columns" stencil. The reference has rows only.
    :meth:`integrate` returns a float32 CUDA tensor ``(n, n)``.
    """

    def __init__(self, n: int, pixel_scale: float, layer_r0: Sequence[float],
                 layer_L0: Sequence[float], layer_wind: Sequence[Tuple[float, float]],
                 layer_altitude_los: Sequence[float],
                 field_of_view_pix: Union[float, Sequence[float]] = 0.0,
                 stencil_rows: int = 2, interp: str = "cubic",
                 lgs_altitude_los: Optional[float] = None, device: str = "gpu",
                 dtype: Any = "float32", seeds: Optional[Sequence[Any]] = None,
                 tau_boil: Optional[Sequence[float]] = None, boil_seed: Optional[Any] = None,
                 host_noise=None, extrude_form: str = "fp32", stencil_columns: int = 0,
                 sparse_depth: Optional[int] = None) -> None:
        config = ExtrusionConfig.create(
            n, pixel_scale, layer_r0, layer_L0, layer_wind, layer_altitude_los,
            field_of_view_pix, stencil_rows, interp, lgs_altitude_los, device, dtype, seeds,
            tau_boil, boil_seed)
        self.config = config
        self.n = config.grid.n
        self.dx = config.grid.pixel_scale
        self.device = config.grid.device
        self.dtype = config.grid.dtype
        self.interp = config.interp
        self.m = config.stencil_rows
        L = len(config.layer_r0)
        if config.lgs_altitude_los is not None:
            mags = [1.0 - a / config.lgs_altitude_los for a in config.layer_altitude_los]
        else:
            mags = [1.0] * L
        extents, spans = [], []
        for (vx, vy), mag, fov in zip(config.layer_wind, mags, config.field_of_view_pix):
            e, s = along_extent_and_span(self.n, vx, vy, mag, fov)
            extents.append(e)
            spans.append(s)
        self.width = int(np.ceil(2.0 * max(extents) + 2.0 * max(config.field_of_view_pix))) + 4
        W = self.width
        if (not isinstance(stencil_columns, (int, np.integer)) or isinstance(stencil_columns, bool)
                or stencil_columns < 0):
            raise ValueError("stencil_columns must be a non-negative integer")
        self.sparse = sparse_points(W, self.m, int(stencil_columns), sparse_depth)
        history = max([0] + [d for d, _ in self.sparse])
        self.capacity = max(spans) + self.n + self.m + 32 + history
        self._tau = [float(t) for t in config.tau_boil]
        self.boiling = any(np.isfinite(t) for t in self._tau)
        if self.boiling and self.sparse:
            raise ValueError("boiling supports the rows-only stencil (stencil_columns=0)")

        # one FP64 device build per distinct outer scale; the reference's
        # eigen-square-root B in the parity mode, the build's Cholesky factor
        # otherwise (the same conditional covariance)
        op_index: dict = {}
        ops = []
        groups = []
        for L0 in config.layer_L0:
            key = round(float(L0), 9)
            if key not in op_index:
                op_index[key] = len(ops)
                # FP32 form: the operator as it is plus the low-order anchor
                # (float64 twin needed for its tables); bf16x3: the increment
                # form, whose small products keep the bf16 terms' rounding
                # small (measured 14x closer to float64 than the plain form)
                ops.append(build_operator(W, self.m, self.dx, float(L0), self.sparse,
                                          b_factor="eigh" if host_noise is not None
                                          else "cholesky", want_seed=self.boiling,
                                          want_float64=extrude_form == "fp32",
                                          want_lo=extrude_form == "fp32" and bool(self.sparse),
                                          increments=extrude_form == "bf16x3"))
            groups.append(op_index[key])
        streams = [NoiseStream(s, host_noise) for s in config.seeds]
        self._streams = streams
        self.layers: List[_LayerGeom] = []
        for (vx, vy), alt, mag, fov in zip(config.layer_wind, config.layer_altitude_los, mags,
                                           config.field_of_view_pix):
            self.layers.append(_LayerGeom(self.n, W, self.dx, vx, vy, alt, self.m, mag, fov,
                                          history))
        bscale = [float(r0) ** (-5.0 / 6.0) for r0 in config.layer_r0]
        torch = torch_module()
        # a sparse stencil feeds single pixels of old rows back into new ones
        # (a longer memory for rounding errors): 64 anchored modes and the
        # operator correction there, 32 modes for the rows-only stencil
        anchor, lo = None, None
        modes = anchor_modes(W, self.sparse)
        if extrude_form == "fp32" and modes:
            anchor = AnchorTables(ops, modes)
        if extrude_form == "fp32" and self.sparse:
            lo = torch.stack([op.Mlo for op in ops])
        self._ring = RingExtruder(W, self.m, self.capacity, [], groups, bscale, streams,
                                  device_operator=torch.stack([op.M for op in ops]),
                                  form=extrude_form, sparse=self.sparse, anchor=anchor,
                                  operator_lo=lo, increments=extrude_form == "bf16x3")
        for op in ops:  # the float64 twins were needed for the anchor only
            op.M64 = None
        # seed each ring with a von Karman screen from the layer's own stream:
        # a W x W screen for the rows-only stencil (as the reference), a taller
        # one cropped to W columns when sparse points need older rows
        side = W if not self.sparse else _smooth_size(max(W, max(spans) + history))
        for i, (r0, L0) in enumerate(zip(config.layer_r0, config.layer_L0)):
            gen = PhaseScreen(n=side, pixel_scale=self.dx, r0=float(r0), L0=float(L0),
                              _stream=streams[i], host_noise=host_noise)
            init = gen.generate()
            ly = self.layers[i]
            self._ring.seed_rows(i, init[: ly.span + ly.history, :W])
            del gen
        # boiling (src/pyturb/extrude.py:472-496, 586-650, 695-753)
        if self.boiling:
            self._boil_layers = [i for i, t in enumerate(self._tau) if np.isfinite(t)]
            self._host_boil = host_noise is not None
            self._boil = NoiseStream(config.boil_seed, host_noise)
            self._S = torch.stack([op.S for op in ops])          # (G, mW, mW)
            self._groups = groups
            self._bscale = bscale
            self._queues = [_RowQueue(self._host_boil) for _ in self._boil_layers]
            self._scratch = RingExtruder(
                W, self.m, self.capacity + self.m, [], [groups[i] for i in self._boil_layers],
                [bscale[i] for i in self._boil_layers], self._queues,
                device_operator=self._ring.M, form=extrude_form, anchor=self._ring.anchor,
                increments=self._ring.increments)

    @property
    def _buf(self):
        return self._ring.buf

    def _plan(self, ly: _LayerGeom) -> int:
        """Rows the layer needs to cover its travel, with the reference's
        compaction bookkeeping applied (``src/pyturb/extrude.py:424-449``)."""
        top = int(np.ceil(ly.along_max + ly.fov + ly.travel)) + 2
        count = 0
        while ly.base + ly.fill - 1 < top:
            if ly.fill == self.capacity:
                ly.base, ly.fill = compact_bounds(ly.base, ly.fill, self._ring.depth,
                                                  ly.along_min - ly.fov + ly.travel)
            ly.fill += 1
            count += 1
        return count

    def set_time(self, t: float) -> None:
        """Advance every layer to time ``t`` (``src/pyturb/extrude.py:656-659``)."""
        counts = []
        for ly in self.layers:
            travel = ly.speed * t / self.dx
            if travel < ly.travel:
                raise ValueError("wind travel is monotonic; travel cannot decrease")
            ly.travel = float(travel)
            counts.append(self._plan(ly))
        self._ring.extrude(counts)

    def boil_step(self, dt: float) -> None:
        """One AR(1) boiling step (``src/pyturb/extrude.py:715-753``): every
        boiling layer's readable rows ``[lo, hi)`` become ``a buf + b fresh``,
        ``a = exp(-dt/tau)``, with ``fresh`` an independent window seeded by
        ``S white`` and extruded with the layer's own operator. With host noise
        the boil stream is consumed in the reference's order (per layer: the
        ``m W`` seed normals, then ``W`` per extruded row)."""
        if not self.boiling:
            return
        torch = torch_module()
        W, m, cap = self.width, self.m, self.capacity
        regions = []
        for q, i in enumerate(self._boil_layers):
            ly = self.layers[i]
            a = float(np.exp(-dt / self._tau[i]))
            b = float(np.sqrt(max(0.0, 1.0 - a * a)))
            lo = max(0, int(np.floor(ly.along_min + ly.travel)) - ly.base - 3)
            hi = ly.fill
            if hi > lo:
                regions.append((q, i, lo, hi, a, b))
        if not regions:
            return
        scr = self._scratch
        scales = np.asarray([self._bscale[i] for _, i, *_ in regions], dtype=np.float32)
        dev = scr.buf.device
        if self._host_boil:
            whites = []
            for (q, i, lo, hi, a, b), sc in zip(regions, scales):
                whites.append(self._boil.draw((m * W,)) * float(sc))
                self._queues[q].rows = [self._boil.draw((W,)) for _ in range(m, hi - lo)]
            X = upload(np.stack(whites))
        else:
            call = self._boil.next_call()
            X = torch.empty((len(regions), m * W), dtype=torch.float32, device=dev)
            _lib.call("pt_fill_normals", self._boil.key, call, len(regions), m * W,
                      scales.ctypes.data_as(C.POINTER(C.c_float)), dptr(X), stream_handle())
            for q, *_ in regions:  # fresh Philox rows for every step's scratch extrusion
                scr._key[q] = np.uint64((self._boil.key ^ (0x9E3779B97F4A7C15 * (call + 1))
                                         ^ (q + 1) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF)
        # seed rows S_g (r0^-5/6 white) for every region, one GEMM per operator group
        seeds = torch.empty((len(regions), m * W), dtype=torch.float32, device=dev)
        lib = _lib.load()
        for g in sorted({self._groups[i] for _, i, *_ in regions}):
            idx = [k for k, (_, i, *_r) in enumerate(regions) if self._groups[i] == g]
            Xg = X[idx].contiguous()
            out = torch.empty_like(Xg)
            nbytes = int(lib.pt_matmul_nt_workspace_bytes(m * W, m * W, len(idx)))
            work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            _lib.call("pt_matmul_nt", m * W, m * W, len(idx), dptr(self._S[g]), dptr(Xg),
                      dptr(out), dptr(work), nbytes, stream_handle())
            seeds[idx] = out
        counts = np.zeros(scr.S, dtype=np.int32)
        for k, (q, i, lo, hi, a, b) in enumerate(regions):
            h = hi - lo
            scr.seed_rows(q, seeds[k].view(m, W)[:min(m, h)])
            counts[q] = max(0, h - m)
        scr.extrude(counts)
        for q, i, lo, hi, a, b in regions:
            ly = self.layers[i]
            phys0 = (ly.base + lo - ly.v0) % cap
            _lib.call("pt_ring_blend", W, cap, dptr(self._ring.buf[i]), int(phys0), hi - lo,
                      a, b, dptr(scr.buf[q]), stream_handle())

    def readout_params(self, thx: float = 0.0, thy: float = 0.0):
        arr = (_lib.ReadoutLayer * len(self.layers))()
        for i, ly in enumerate(self.layers):
            off_a, off_p = ly.offsets_for_direction(thx, thy)
            p = arr[i]
            p.screen = i
            p.row_max = ly.fill - 1
            p.anchor_phys = (ly.base - ly.v0) % self.capacity
            p.cos_t = ly.cos
            p.sin_t = ly.sin
            p.mag = ly.mag
            p.shift_along = (ly.travel - ly.base) + off_a
            p.shift_perp = off_p
        return arr

    def integrate(self, thx: float = 0.0, thy: float = 0.0, scale: float = 1.0, out=None):
        """Summed phase ``(n, n)`` toward direction tangents (thx, thy)
        (``src/pyturb/extrude.py:754-770``)."""
        torch = torch_module()
        if out is None:
            out = torch.empty((self.n, self.n), dtype=torch.float32, device=self._buf.device)
        params = self.readout_params(thx, thy)
        _lib.call("pt_readout", self.n, self.width, self.capacity, _INTERP[self.interp],
                  len(self.layers), params, dptr(self._buf), float(scale), dptr(out),
                  stream_handle())
        return out

