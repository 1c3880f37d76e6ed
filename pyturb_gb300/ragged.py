"""Ragged Monte-Carlo ensembles: many independent screens of mixed sizes,
outer scales and r0, one native call per (size, pixel scale, L0) group.

The reference draws such an ensemble as independent
``PhaseScreen(n_i, dx_i, r0_i, L0_i).generate()`` calls
(``src/pyturb/fourier.py:98-282``). The filter amplitude is proportional to
``r0^(-5/6)`` (``fourier.py:131-228``), so the screens of one (n, dx, L0) group
share a unit-r0 grid plan and filter and take ``r0_i^(-5/6)`` as a per-screen
factor in the fused column epilogue (``pt_generate_scaled``). The screens are
packed into one float32 buffer, group after group; the groups are spread over
a few streams with a workspace each, so the small groups' latency-bound
launches overlap. :meth:`RaggedEnsemble.screen` returns screen ``i`` in the
caller's order.
"""

from __future__ import annotations

from typing import List, Sequence

import numpy as np

from . import _lib
from .backend import NoiseStream, check_device, cuda_device, dptr, stream_handle, torch_module, upload
from .fourier import Grid, amplitude_table, subharmonic_tables

__all__ = ["RaggedEnsemble"]


class _Group:
    """The screens of one (n, dx, L0): grid plan, unit-r0 filters, r0 factors."""

    def __init__(self, n: int, dx: float, L0: float, P: int, power_law: float,
                 members: List[int], r0: np.ndarray) -> None:
        self.n, self.dx, self.L0 = n, dx, L0
        self.members = members
        freqs, sh_amps = subharmonic_tables(n, dx, 1.0, L0, P, power_law)
        self.grid = Grid(n, dx, freqs, workspace=False)
        self.amplitude = upload(amplitude_table(n, dx, 1.0, L0, power_law))
        self.sh_amp = upload(sh_amps) if P else None
        self.scale = upload(np.asarray([r0[i] ** (-5.0 / 6.0) for i in members],
                                       dtype=np.float32))


class RaggedEnsemble:
    """``len(sizes)`` independent von Karman screens [rad]: screen ``i`` is
    ``sizes[i]`` square at ``pixel_scale`` (scalar or per screen) with Fried
    parameter ``r0[i]`` and outer scale ``L0[i]`` (scalars broadcast), with
    ``subharmonics`` levels of 3x3 low-order modes.

    :meth:`generate` draws a new ensemble (in-kernel Philox keyed by ``seed``,
    a fresh counter per call) into :attr:`buffer`. ``autotune=True`` times
    each group's radix plan or column variant once (cached on disk per
    device, size and batch; see :mod:`pyturb_gb300.tuning`)."""

    def __init__(self, sizes: Sequence[int], r0, L0, pixel_scale=1.0 / 64,
                 subharmonics: int = 3, power_law: float = 11.0 / 3.0, seed=None,
                 device: str = "gpu", streams: int = 4, autotune: bool = False) -> None:
        torch = torch_module()
        check_device(device)
        sizes = np.asarray(sizes, dtype=np.int64).reshape(-1)
        S = int(sizes.size)
        if S < 1:
            raise ValueError("need at least one screen")
        r0 = np.broadcast_to(np.asarray(r0, dtype=np.float64), (S,))
        L0 = np.broadcast_to(np.asarray(L0, dtype=np.float64), (S,))
        dx = np.broadcast_to(np.asarray(pixel_scale, dtype=np.float64), (S,))
        if np.any(sizes < 2) or np.any(sizes > 4096):
            raise ValueError("screen sizes must be in [2, 4096]")
        for name, v in (("r0", r0), ("L0", L0), ("pixel_scale", dx)):
            if not np.all(np.isfinite(v) & (v > 0)):
                raise ValueError(f"{name} must be positive and finite")
        if not isinstance(subharmonics, (int, np.integer)) or not 0 <= subharmonics <= 16:
            raise ValueError("subharmonics must be an integer in [0, 16]")
        self.S, self.sizes, self.P = S, sizes, int(subharmonics)
        keys: dict = {}
        for i in range(S):
            keys.setdefault((int(sizes[i]), float(dx[i]), float(L0[i])), []).append(i)
        self.groups = [_Group(n, d, l0, self.P, float(power_law), members, r0)
                       for (n, d, l0), members in sorted(keys.items())]
        self.offsets = np.zeros(S, dtype=np.int64)
        self._group_off = []
        pos = 0
        for g in self.groups:
            self._group_off.append(pos)
            for i in g.members:
                self.offsets[i] = pos
                pos += int(sizes[i]) ** 2
        dev = cuda_device()
        self.buffer = torch.empty(pos, dtype=torch.float32, device=dev)
        # groups run on `streams` streams (largest groups first, round robin),
        # each stream with its own workspace, so small groups overlap
        if not 1 <= int(streams) <= 16:
            raise ValueError("streams must be in [1, 16]")
        self.work_bytes = max(g.grid.work_bytes for g in self.groups)
        self.n_streams = min(int(streams), len(self.groups))
        self._works = [torch.empty(self.work_bytes, dtype=torch.uint8, device=dev)
                       for _ in range(self.n_streams)]
        self.work = self._works[0]
        self._side = [torch.cuda.Stream(dev) for _ in range(self.n_streams - 1)]
        self._order = sorted(range(len(self.groups)),
                             key=lambda k: -len(self.groups[k].members) * self.groups[k].n ** 2)
        self._rng = NoiseStream(seed, None)
        self._keys = [self._rng.next_key() for _ in self.groups]
        self.tuning = {}
        if autotune:  # per group: radix plan or column variant, cached per (n, batch)
            from .tuning import tune_grid

            for k, g in enumerate(self.groups):
                self.tuning[(g.n, g.dx, g.L0)] = tune_grid(
                    g.grid, lambda k=k: self._launch_group(k, 0, self._works[0],
                                                           torch.cuda.current_stream()),
                    len(g.members), workload="ragged")

    def _launch_group(self, k: int, call: int, work, stream) -> None:
        g, off, key = self.groups[k], self._group_off[k], self._keys[k]
        _lib.call("pt_generate_scaled", g.grid.handle, len(g.members), dptr(g.amplitude),
                  dptr(g.sh_amp), key, call, 0, g.n, 1.0, dptr(g.scale),
                  self.buffer.data_ptr() + 4 * off, dptr(work), self.work_bytes,
                  stream.cuda_stream)

    def generate(self):
        """Draw a new ensemble into :attr:`buffer` and return it (ordered on the
        current stream: later work on it sees the whole ensemble)."""
        torch = torch_module()
        call = self._rng.next_call()
        main = torch.cuda.current_stream()
        streams = [main] + self._side
        for sd in self._side:
            sd.wait_stream(main)
        for slot, k in enumerate(self._order):
            b = slot % self.n_streams
            self._launch_group(k, call, self._works[b], streams[b])
        for sd in self._side:
            main.wait_stream(sd)
        return self.buffer

    def screen(self, i: int):
        """Screen ``i`` as an ``(n_i, n_i)`` view of :attr:`buffer`."""
        n = int(self.sizes[i])
        o = int(self.offsets[i])
        return self.buffer[o:o + n * n].view(n, n)

    @property
    def n_groups(self) -> int:
        return len(self.groups)
