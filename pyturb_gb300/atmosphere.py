"""Layered atmosphere producing pupil OPD on the GB300 (drop-in for ``pyturb.Atmosphere``).

Same constructor, seeding and call surface as ``src/pyturb/atmosphere.py:108-1318``:
:meth:`frames` / :meth:`opd` / :meth:`evolve` (frozen flow, spectral or
extrusion engine), :meth:`sample` (Monte-Carlo), off-axis ``directions``,
the LGS cone, spectral boiling, dispersion-aware OPD conversion. Outputs are
float32 CUDA ``torch.Tensor`` objects.

GB300 layout: the spectral engine keeps every layer's spectrum in one
``(L, ns, ns)`` complex slab; one native call renders a whole batch of
frames (each frame's layer sum, inverse FFT, subharmonics, crop and OPD scale
fused into two shared-memory passes), so :meth:`frames` computes frames in
chunks of up to ``frames_chunk`` and yields views of them. Without boiling,
frames at different times are independent (the reference evaluates each frame
from the fixed spectra at its own ``t``), so batching changes nothing but
speed; with boiling each frame depends on the previous boiling step and is
rendered one at a time.
"""

from __future__ import annotations

import warnings
from typing import Any, Dict, Iterator, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .backend import NoiseStream, dptr, stream_handle, torch_module, upload
from .config import AtmosphereConfig
from .flow import SpectralLayers
from .fourier import PhaseScreen, amplitude_table, subharmonic_tables
from .optics import ARCSEC_TO_RAD, output_scale, seeing_from_r0
from .profiles import Layer

__all__ = ["Atmosphere", "FrameLoop", "PeriodicWrapWarning", "ExtrudeBoilingPerformanceWarning"]


class PeriodicWrapWarning(UserWarning):
    """The periodic spectral screen has wrapped (``src/pyturb/atmosphere.py:55-66``)."""


class ExtrudeBoilingPerformanceWarning(UserWarning):
    """Boiling on the extrusion engine re-extrudes a fresh window per step
    (``src/pyturb/atmosphere.py:69-85``)."""


def catmull_rom_weights(t):
    """Catmull-Rom weights of taps (-1, 0, 1, 2) at fraction t (``src/pyturb/extrude.py:74-83``)."""
    t2 = t * t
    t3 = t2 * t
    return (0.5 * (-t + 2.0 * t2 - t3), 0.5 * (2.0 - 5.0 * t2 + 3.0 * t3),
            0.5 * (t + 4.0 * t2 - 3.0 * t3), 0.5 * (-t2 + t3))


def lanczos_weights(t, a: int = 3):
    """Normalised Lanczos-a taps (-a+1 .. a) at fraction t (``src/pyturb/infinite.py:67-85``)."""
    offsets = tuple(range(-a + 1, a + 1))
    raw = [np.sinc(t - d) * np.sinc((t - d) / a) for d in offsets]
    total = raw[0]
    for r in raw[1:]:
        total = total + r
    return offsets, tuple(r / total for r in raw)


class Atmosphere:
    """A multi-layer turbulent atmosphere producing pupil OPD.

    Parameters are those of the reference (``src/pyturb/atmosphere.py:305-328``)
    plus ``host_noise`` (parity mode, see :class:`pyturb_gb300.PhaseScreen`)
    and ``frames_chunk`` (frames rendered per native call in :meth:`frames`).
    """

    def __init__(self, layers: Sequence[Layer], r0: Optional[float] = None,
                 seeing: Optional[float] = None, wavelength: float = 500e-9,
                 zenith_angle: float = 0.0, diameter: float = 8.0, n: int = 512,
                 L0: Optional[float] = None, power_law: float = 11.0 / 3.0,
                 inner_scale: float = 0.0, subharmonics: int = 8, field_of_view: float = 0.0,
                 tau_boil=None, engine: str = "spectral", interp: str = "cubic",
                 lgs_altitude: Optional[float] = None, dispersion: Optional[str] = None,
                 wet_fraction: float = 0.0, device: str = "gpu", dtype: str = "float32",
                 seed: Optional[int] = None, host_noise=None, frames_chunk: int = 64) -> None:
        config = AtmosphereConfig.create(
            layers, r0, seeing, wavelength, zenith_angle, diameter, n, L0, power_law,
            inner_scale, subharmonics, field_of_view, tau_boil, engine, interp, lgs_altitude,
            dispersion, wet_fraction, device, dtype, seed)
        if config.engine == "extrude" and config.has_tau_boil:
            warnings.warn(
                "boiling (tau_boil) on engine='extrude' re-extrudes an independent fresh "
                "screen every step and is markedly slower than the spectral engine's "
                "per-mode AR(1) boiling.", ExtrudeBoilingPerformanceWarning, stacklevel=2)
        self.config = config
        self.engine = config.engine
        self.interp = config.interp
        self.lgs_altitude = config.lgs_altitude
        self.dispersion = config.dispersion
        self.wet_fraction = config.wet_fraction
        self.wavelength = config.wavelength
        self.r0_zenith = config.r0_zenith
        self.zenith_angle = config.zenith_angle
        self.diameter = config.diameter
        self.n = config.grid.n
        self.subharmonics = config.subharmonics
        self.power_law = config.power_law
        self.inner_scale = config.inner_scale
        self.field_of_view = config.field_of_view
        self.device = config.grid.device
        self.dtype = config.grid.dtype.name
        self.pixel_scale = config.grid.pixel_scale
        self.frames_chunk = max(1, int(frames_chunk))
        self._host_noise = host_noise

        cos_z = np.cos(np.deg2rad(self.zenith_angle))
        self.airmass = 1.0 / cos_z
        self.r0_los = self.r0_zenith * cos_z ** (3.0 / 5.0)
        self.layers = [ly.to_layer() for ly in config.layers]

        max_alt_los = max(ly.altitude for ly in self.layers) * self.airmass
        margin_m = max_alt_los * np.tan(self.field_of_view * ARCSEC_TO_RAD)
        self.margin_pix = int(np.ceil(margin_m / self.pixel_scale))
        self.n_screen = self.n + 2 * self.margin_pix
        self._screen_period_m = self.n_screen * self.pixel_scale
        self._wrap_warned = False
        self.tau_boil = np.asarray(config.tau_boil, dtype=np.float64)

        # Seeding mirrors src/pyturb/atmosphere.py:393-470 spawn for spawn, so a
        # parity run (host_noise) consumes exactly the reference's streams.
        self.seed = config.seed
        master = np.random.SeedSequence(self.seed)
        children = master.spawn(len(self.layers))
        self._boil_seed = int(master.spawn(1)[0].generate_state(1)[0])
        self._ext_boil_seed = int(master.spawn(1)[0].generate_state(1)[0])
        self._boil_rng = NoiseStream(self._boil_seed, host_noise)
        self._r0_layers, self._gen_seeds, self._flow_seeds, ext_seeds = [], [], [], []
        self._vx, self._vy, self._alt = [], [], []
        for ly, child in zip(self.layers, children):
            r0_i = self.r0_los * ly.cn2_fraction ** (-3.0 / 5.0)
            gen_seed, flow_seed, ext_seed = child.spawn(3)
            self._r0_layers.append(r0_i)
            self._gen_seeds.append(int(gen_seed.generate_state(1)[0]))
            self._flow_seeds.append(int(flow_seed.generate_state(1)[0]))
            ext_seeds.append(int(ext_seed.generate_state(1)[0]))
            vx, vy = ly.wind_vector
            self._vx.append(vx)
            self._vy.append(vy)
            self._alt.append(ly.altitude * self.airmass)
        self._vx = np.asarray(self._vx, dtype=np.float64)
        self._vy = np.asarray(self._vy, dtype=np.float64)
        self._alt = np.asarray(self._alt, dtype=np.float64)

        groups: Dict[float, List[int]] = {}
        for i, ly in enumerate(self.layers):
            groups.setdefault(round(float(ly.L0), 9), []).append(i)
        self._sample_specs = []  # (r0, L0, seed) per L0 group
        for idxs, child in zip(groups.values(), master.spawn(len(groups))):
            if len(idxs) == 1:
                i = idxs[0]
                self._sample_specs.append((self._r0_layers[i], self.layers[i].L0,
                                           self._gen_seeds[i]))
                continue
            r0_agg = sum(self._r0_layers[i] ** (-5.0 / 3.0) for i in idxs) ** (-3.0 / 5.0)
            self._sample_specs.append((r0_agg, self.layers[idxs[0]].L0,
                                       int(child.generate_state(1)[0])))
        self._sample_generators: Optional[List[PhaseScreen]] = None

        self._lgs_mag = None
        if self.lgs_altitude is not None:
            lgs_los = self.lgs_altitude * self.airmass
            mag = 1.0 - self._alt / lgs_los
            if np.any(mag <= 0.0):
                raise ValueError(
                    f"lgs_altitude ({self.lgs_altitude:.0f} m) must exceed every layer "
                    "altitude (projected to the line of sight): a degenerate (<= 0) cone "
                    "magnification is rejected on both engines.")
            if self.engine == "spectral":
                self._lgs_mag = mag

        self._t = 0.0
        if self.engine == "spectral":
            self._build_spectral()
        else:
            from .extrude import ExtrudedAtmosphere

            fov_pix = [a * np.tan(self.field_of_view * ARCSEC_TO_RAD) / self.pixel_scale
                       for a in self._alt]
            self._ext_kwargs = dict(
                n=self.n, pixel_scale=self.pixel_scale, layer_r0=self._r0_layers,
                layer_L0=[ly.L0 for ly in self.layers],
                layer_wind=list(zip(self._vx, self._vy)), layer_altitude_los=list(self._alt),
                field_of_view_pix=fov_pix, interp=self.interp,
                lgs_altitude_los=(None if self.lgs_altitude is None
                                  else self.lgs_altitude * self.airmass),
                device=self.device, dtype=self.dtype, seeds=ext_seeds,
                tau_boil=(None if not config.has_tau_boil else list(self.tau_boil)),
                boil_seed=self._ext_boil_seed, host_noise=host_noise)
            self._ext = ExtrudedAtmosphere(**self._ext_kwargs)

    # ------------------------------------------------------------------ spectral state
    def _build_spectral(self) -> None:
        """Stacked layer spectra + subharmonics (``src/pyturb/atmosphere.py:532-579``)."""
        ns, dx, P = self.n_screen, self.pixel_scale, self.subharmonics
        amps, sh_amps, freqs = [], [], None
        for r0_i, ly in zip(self._r0_layers, self.layers):
            amps.append(amplitude_table(ns, dx, r0_i, ly.L0, self.power_law, self.inner_scale))
            f, a = subharmonic_tables(ns, dx, r0_i, ly.L0, P, self.power_law, self.inner_scale)
            freqs = f
            sh_amps.append(a)
        self._amplitudes_host = np.stack(amps)
        sh = np.stack(sh_amps, axis=1) if P else np.zeros((0, len(self.layers), 3, 3))
        self._sh_freqs = freqs if P else np.zeros((0, 3))
        streams = [NoiseStream(s, self._host_noise) for s in self._flow_seeds]
        self._spec = SpectralLayers(ns, dx, self._sh_freqs, self._amplitudes_host, sh, streams)
        self._boiling = bool(np.any(np.isfinite(self.tau_boil)))
        self._spec_initial = None
        if self._boiling:
            self._spec_initial = (self._spec.spectra.clone(), self._spec.sh_coef.clone())
            main_tau, sh_tau = self._boil_tau_maps()
            self._main_tau = upload(main_tau)
            self._sh_tau = upload(sh_tau) if P else None
        if self._lgs_mag is not None:
            self._build_lgs_zoom()

    def _boil_tau_maps(self) -> Tuple[np.ndarray, np.ndarray]:
        """Per-mode boiling times ``tau(f) = tau_boil (f/f_ref)^(-2/3)`` clamped below
        ``f_ref`` (``src/pyturb/atmosphere.py:618-658``)."""
        L0s = np.array([ly.L0 for ly in self.layers], dtype=np.float64)
        df = 1.0 / (self.n_screen * self.pixel_scale)
        f_ref = np.where(np.isfinite(L0s), 1.0 / np.where(L0s > 0, L0s, np.inf), df)
        f = np.fft.fftfreq(self.n_screen, d=self.pixel_scale)
        fr = np.hypot(f[:, None], f[None, :])
        ratio = np.clip(fr[None] / f_ref[:, None, None], 1.0, None)
        main = self.tau_boil[:, None, None] * ratio ** (-2.0 / 3.0)
        if not self.subharmonics:
            return main, np.zeros(0)
        fp = self._sh_freqs
        fr_sh = np.hypot(fp[:, :, None], fp[:, None, :])
        ratio_sh = np.clip(fr_sh[:, None] / f_ref[None, :, None, None], 1.0, None)
        return main, self.tau_boil[None, :, None, None] * ratio_sh ** (-2.0 / 3.0)

    def _build_lgs_zoom(self) -> None:
        """Per-layer cone-zoom taps (``src/pyturb/atmosphere.py:581-616``)."""
        centre = (self.n_screen - 1) / 2.0
        base = np.arange(self.n, dtype=np.float64) - (self.n - 1) / 2.0
        idx_l, w_l = [], []
        for mag in self._lgs_mag:
            pos = centre + base * float(mag)
            p0 = np.floor(pos).astype(np.int64)
            fr = pos - p0
            if self.interp == "linear":
                offsets, weights = (0, 1), (1.0 - fr, fr)
            elif self.interp == "lanczos":
                offsets, weights = lanczos_weights(fr)
            else:
                offsets, weights = (-1, 0, 1, 2), catmull_rom_weights(fr)
            idx_l.append(np.stack([np.clip(p0 + o, 0, self.n_screen - 1) for o in offsets]))
            w_l.append(np.stack([np.asarray(w) for w in weights]))
        self._zoom_idx = upload(np.stack(idx_l).astype(np.int32), dtype=torch_module().int32)
        self._zoom_w = upload(np.stack(w_l))
        self._zoom_taps = len(idx_l[0])

    # ------------------------------------------------------------------ properties
    @property
    def r0(self) -> float:
        return self.r0_los

    @property
    def seeing(self) -> float:
        return seeing_from_r0(self.r0_los, self.wavelength)

    @property
    def time(self) -> float:
        return self._t

    @property
    def time_to_wrap(self) -> float:
        if self.engine != "spectral":
            return float("inf")
        speeds = np.array([ly.wind_speed for ly in self.layers])
        with np.errstate(divide="ignore"):
            periods = self._screen_period_m / speeds
        finite = periods[np.isfinite(periods)]
        return float(finite.min()) if finite.size else float("inf")

    def _check_wrap(self, disp_x: np.ndarray, disp_y: np.ndarray) -> None:
        disp = np.hypot(np.asarray(disp_x), np.asarray(disp_y))
        wrapped = disp > self._screen_period_m
        if not np.any(wrapped):
            return
        self._wrap_warned = True
        flat = np.argwhere(wrapped)[0]
        idx = int(flat[-1])
        ly = self.layers[idx]
        warnings.warn(
            f"engine='spectral' layer {idx} (altitude={ly.altitude:.0f} m, "
            f"wind_speed={ly.wind_speed:.1f} m/s) has wrapped: its cumulative travel "
            f"({float(disp[tuple(flat)]):.2f} m) exceeds the screen's period "
            f"({self._screen_period_m:.2f} m).", PeriodicWrapWarning, stacklevel=3)

    def _scale(self, wavelength: Optional[float]) -> float:
        return output_scale(self.wavelength, wavelength, self.dispersion, self.wet_fraction)

    # ------------------------------------------------------------------ rendering
    def _spectral_frames(self, times: np.ndarray, oxs: np.ndarray, oys: np.ndarray,
                         scale: float):
        """Frames for (t, ox, oy) triples: (F, n, n), each ``_integrate`` of the reference."""
        disp_x = self._vx[None, :] * times[:, None] + self._alt[None, :] * oxs[:, None]
        disp_y = self._vy[None, :] * times[:, None] + self._alt[None, :] * oys[:, None]
        if not self._wrap_warned:
            self._check_wrap(disp_x, disp_y)
        if self._lgs_mag is not None:
            torch = torch_module()
            out = torch.empty((len(times), self.n, self.n), dtype=torch.float32,
                              device=self._spec.grid.device)
            for k in range(len(times)):
                screens = self._spec.layer_screens(disp_x[k], disp_y[k])
                _lib.call("pt_lgs_zoom", len(self.layers), self.n_screen, self.n,
                          self._zoom_taps, dptr(self._zoom_idx), dptr(self._zoom_w),
                          dptr(screens), float(scale), dptr(out[k]), stream_handle())
            return out
        return self._spec.frames(disp_x, disp_y, self.margin_pix, self.n, scale)

    def _phase_frames(self, times, oxs, oys, scale: float):
        if self.engine == "spectral":
            return self._spectral_frames(np.asarray(times, dtype=np.float64),
                                         np.asarray(oxs, dtype=np.float64),
                                         np.asarray(oys, dtype=np.float64), scale)
        torch = torch_module()
        outs = []
        for t, ox, oy in zip(times, oxs, oys):
            self._ext.set_time(float(t))
            outs.append(self._ext.integrate(float(ox), float(oy), scale=scale))
        return torch.stack(outs)

    def _boil_step(self, dt: float) -> None:
        """One AR(1) step per Fourier mode (``src/pyturb/atmosphere.py:1092-1126``)."""
        with np.errstate(divide="ignore"):
            alpha = np.where(np.isfinite(self.tau_boil), np.exp(-dt / self.tau_boil), 1.0)
        if np.all(alpha >= 1.0):
            return
        L, ns, P = len(self.layers), self.n_screen, self.subharmonics
        noise = sh_noise = None
        if self._boil_rng.injected:
            noise = upload(self._boil_rng.draw((2, L, ns, ns)))
            if P:
                sh_noise = upload(self._boil_rng.draw((2, P, L, 3, 3)))
        call = self._boil_rng.next_call()
        sp = self._spec
        _lib.call("pt_boil_step", sp.grid.handle, L, dptr(sp.spectra),
                  dptr(sp.sh_coef) if P else None, dptr(sp.amplitude), dptr(sp.sh_amp),
                  dptr(self._main_tau), dptr(self._sh_tau), float(dt), dptr(noise),
                  dptr(sh_noise), self._boil_rng.key, call, stream_handle())

    def _after_step(self, dt: float) -> None:
        if self.engine == "spectral":
            self._boil_step(dt)
        else:
            self._ext.boil_step(dt)

    # ------------------------------------------------------------------ public API
    def opd(self, t: float = 0.0, directions: Optional[Sequence[Tuple[float, float]]] = None,
            wavelength: Optional[float] = None):
        """OPD [m] (or phase at ``wavelength``) at time ``t``
        (``src/pyturb/atmosphere.py:801-869``)."""
        scale = self._scale(wavelength)
        if directions is None:
            return self._phase_frames([float(t)], [0.0], [0.0], scale)[0]
        oxs, oys = [], []
        for thx, thy in directions:
            radius = float(np.hypot(thx, thy))
            if radius > self.field_of_view:
                raise ValueError(
                    f"direction ({thx}, {thy}) arcsec has radius {radius:.3g} arcsec, "
                    f"exceeding the declared field_of_view={self.field_of_view} arcsec. "
                    "Construct the Atmosphere with a field_of_view covering every "
                    "direction you plan to request.")
            oxs.append(np.tan(thx * ARCSEC_TO_RAD))
            oys.append(np.tan(thy * ARCSEC_TO_RAD))
        times = [float(t)] * len(oxs)
        return self._phase_frames(times, oxs, oys, scale)

    def frames(self, dt: float, steps: int,
               wavelength: Optional[float] = None) -> Iterator[Tuple[float, Any]]:
        """Yield ``(t, opd)`` for ``steps`` frames spaced by ``dt``
        (``src/pyturb/atmosphere.py:1128-1154``)."""
        if dt <= 0:
            raise ValueError("dt must be positive")
        if steps < 1:
            raise ValueError("steps must be >= 1")
        dt = float(dt)
        scale = self._scale(wavelength)
        steps = int(steps)
        batched = self.engine == "spectral" and not self._boiling
        if not batched:
            for _ in range(steps):
                t = self._t
                frame = self._phase_frames([t], [0.0], [0.0], scale)[0]
                yield t, frame
                self._t += dt
                self._after_step(dt)
            return
        done = 0
        while done < steps:
            k = min(self.frames_chunk, steps - done)
            times = np.empty(k)
            t = self._t
            for i in range(k):  # the reference's clock: repeated float additions
                times[i] = t
                t += dt
            chunk = self._phase_frames(times, np.zeros(k), np.zeros(k), scale)
            for i in range(k):
                yield float(times[i]), chunk[i]
                self._t = float(times[i]) + dt
            done += k

    def frames_host(self, dt: float, steps: int, wavelength: Optional[float] = None, out=None):
        """All ``steps`` frames of :meth:`frames` delivered into host memory.

        Returns a pinned CPU tensor ``(steps, n, n)`` (or fills ``out``, which
        should be pinned for the copies to overlap). Chunks of ``frames_chunk``
        frames are rendered into two alternating device buffers and copied to
        the host on a side stream while the next chunk renders, so the run is
        bounded by the slower of the GPU and the device-to-host link. Advances
        the clock exactly as iterating :meth:`frames` does.
        """
        if dt <= 0:
            raise ValueError("dt must be positive")
        if steps < 1:
            raise ValueError("steps must be >= 1")
        torch = torch_module()
        steps = int(steps)
        if out is None:
            out = torch.empty((steps, self.n, self.n), dtype=torch.float32, pin_memory=True)
        if self.engine != "spectral" or self._boiling or self._lgs_mag is not None:
            for i, (_t, f) in enumerate(self.frames(dt, steps, wavelength)):
                out[i].copy_(f)
            return out
        dev = self._spec.grid.device
        k = self.frames_chunk
        bufs = [torch.empty((k, self.n, self.n), dtype=torch.float32, device=dev)
                for _ in range(2)]
        done_copy = [None, None]
        main = torch.cuda.current_stream(dev)
        side = torch.cuda.Stream(dev)
        dt = float(dt)
        t = self._t
        for c, start in enumerate(range(0, steps, k)):
            m = min(k, steps - start)
            times = np.empty(m)
            for i in range(m):  # the reference's clock: repeated float additions
                times[i] = t
                t += dt
            b = c % 2
            if done_copy[b] is not None:
                main.wait_event(done_copy[b])
            self.render(times, wavelength, out=bufs[b][:m])
            ready = torch.cuda.Event()
            ready.record(main)
            with torch.cuda.stream(side):
                side.wait_event(ready)
                out[start:start + m].copy_(bufs[b][:m], non_blocking=True)
                done_copy[b] = torch.cuda.Event()
                done_copy[b].record(side)
        side.synchronize()
        self._t = t
        return out

    def render(self, times: Sequence[float], wavelength: Optional[float] = None, out=None):
        """All on-axis frames at ``times`` in one call, ``(F, n, n)`` — each equal to
        ``opd(t)`` (spectral engine, frozen flow, no LGS). ``out`` may be a
        preallocated float32 CUDA tensor of that shape."""
        if self.engine != "spectral" or self._boiling or self._lgs_mag is not None:
            raise ValueError("render() needs the spectral engine without boiling or LGS")
        t = np.asarray(times, dtype=np.float64).reshape(-1)
        disp_x = self._vx[None, :] * t[:, None]
        disp_y = self._vy[None, :] * t[:, None]
        if not self._wrap_warned:
            self._check_wrap(disp_x, disp_y)
        return self._spec.frames(disp_x, disp_y, self.margin_pix, self.n,
                                 self._scale(wavelength), out=out)

    def frame_loop(self, dt: float, steps: int, wavelength: Optional[float] = None,
                   branches=4) -> "FrameLoop":
        """A :class:`FrameLoop`: the ``steps``-frame loop of :meth:`frames` at
        spacing ``dt`` captured once as a CUDA graph, replayed at any start time
        (spectral engine, frozen flow, no LGS). ``branches="auto"`` times 1-4
        concurrent branches once (cached on disk per device and sizes)."""
        if branches == "auto":
            from .tuning import choose

            loop = FrameLoop(self, dt, steps, wavelength, 1)
            choose(f"frame_loop|branches|ns={self.n_screen}|L={len(self.layers)}|"
                   f"steps={int(steps)}|chunk={self.frames_chunk}", [1, 2, 3, 4],
                   loop.capture, lambda: loop.render(0.0), warmup=1, reps=3)
            return loop
        return FrameLoop(self, dt, steps, wavelength, branches)

    def evolve(self, dt: float, wavelength: Optional[float] = None):
        """Advance the clock by ``dt`` and return the new OPD
        (``src/pyturb/atmosphere.py:1156-1189``)."""
        if dt <= 0:
            raise ValueError("dt must be positive")
        self._t += float(dt)
        self._after_step(float(dt))
        return self._phase_frames([self._t], [0.0], [0.0], self._scale(wavelength))[0]

    def _generators(self) -> List[PhaseScreen]:
        if self._sample_generators is None:
            self._sample_generators = [
                PhaseScreen(n=self.n_screen, pixel_scale=self.pixel_scale, r0=r0_g, L0=L0_g,
                            subharmonics=self.subharmonics, power_law=self.power_law,
                            inner_scale=self.inner_scale, seed=seed_g,
                            host_noise=self._host_noise)
                for r0_g, L0_g, seed_g in self._sample_specs]
        return self._sample_generators

    def sample(self, count: Optional[int] = None, wavelength: Optional[float] = None):
        """Independent integrated OPDs, one aggregate screen per L0 group
        (``src/pyturb/atmosphere.py:1191-1219``)."""
        squeeze = count is None
        c = 1 if squeeze else int(count)
        if c < 1:
            raise ValueError("count must be >= 1")
        torch = torch_module()
        scale = self._scale(wavelength)
        gens = self._generators()
        out = torch.empty((c, self.n, self.n), dtype=torch.float32, device=gens[0]._grid.device)
        for g, gen in enumerate(gens):
            gen._generate_into(out, c, self.margin_pix, self.n, scale, accumulate=g > 0)
        return out[0] if squeeze else out

    def sample_host(self, count: int, wavelength: Optional[float] = None, out=None,
                    chunk: int = 64):
        """``count`` independent OPDs delivered into host memory.

        Returns a pinned CPU tensor ``(count, n, n)`` (or fills ``out``, which
        should be pinned for the copies to overlap). Chunks of ``chunk``
        screens are drawn into two alternating device buffers and copied to the
        host on a side stream while the next chunk draws; each chunk is one
        :meth:`sample` call, so the screens are those of repeated
        ``sample(chunk)`` calls (the last one shorter)."""
        count, chunk = int(count), int(chunk)
        if count < 1:
            raise ValueError("count must be >= 1")
        if chunk < 1:
            raise ValueError("chunk must be >= 1")
        torch = torch_module()
        if out is None:
            out = torch.empty((count, self.n, self.n), dtype=torch.float32, pin_memory=True)
        scale = self._scale(wavelength)
        gens = self._generators()
        dev = gens[0]._grid.device
        k = min(chunk, count)
        bufs = [torch.empty((k, self.n, self.n), dtype=torch.float32, device=dev)
                for _ in range(2)]
        done_copy = [None, None]
        main = torch.cuda.current_stream(dev)
        side = torch.cuda.Stream(dev)
        for c, start in enumerate(range(0, count, k)):
            m = min(k, count - start)
            b = c % 2
            if done_copy[b] is not None:
                main.wait_event(done_copy[b])
            for g, gen in enumerate(gens):
                gen._generate_into(bufs[b], m, self.margin_pix, self.n, scale, accumulate=g > 0)
            ready = torch.cuda.Event()
            ready.record(main)
            with torch.cuda.stream(side):
                side.wait_event(ready)
                out[start:start + m].copy_(bufs[b][:m], non_blocking=True)
                done_copy[b] = torch.cuda.Event()
                done_copy[b].record(side)
        side.synchronize()
        return out

    def reset(self) -> "Atmosphere":
        """Back to ``t = 0`` with the initial turbulence (``src/pyturb/atmosphere.py:1221-1243``)."""
        self._t = 0.0
        self._wrap_warned = False
        if self.engine == "extrude":
            from .extrude import ExtrudedAtmosphere

            self._ext = ExtrudedAtmosphere(**self._ext_kwargs)
        elif self._boiling:
            self._boil_rng = NoiseStream(self._boil_seed, self._host_noise)
            s0, c0 = self._spec_initial
            self._spec.spectra.copy_(s0)
            self._spec.sh_coef.copy_(c0)
        return self

    def __repr__(self) -> str:
        return (f"Atmosphere(layers={len(self.layers)}, r0={self.r0_los:.3f} m, "
                f"seeing={self.seeing:.2f}\", n={self.n}, diameter={self.diameter} m, "
                f"engine={self.engine!r}, device={self.device!r})")


class FrameLoop:
    """The frame loop of :meth:`Atmosphere.frames` captured as a CUDA graph.

    The graph holds the chunked frame-synthesis launches for the relative
    times ``0, dt, 2 dt, ...`` (the reference's clock of repeated additions,
    ``src/pyturb/atmosphere.py:1128-1154``), reading a translated copy of the
    layer state. :meth:`render` moves the stored spectra and subharmonic
    coefficients to ``t0`` with one exact phase-ramp launch
    (``pt_layers_translate``) and replays the graph, so a window of frames at
    any start time costs two launches from the host. The frames equal
    ``Atmosphere.render(t0 + relative times)`` to float32 rounding. The layer
    state is read at replay time, so re-seeding the atmosphere between
    replays renders new realisations of the same window.
    """

    def __init__(self, atm: "Atmosphere", dt: float, steps: int,
                 wavelength: Optional[float] = None, branches: int = 4) -> None:
        torch = torch_module()
        if not 1 <= int(branches) <= 8:
            raise ValueError("branches must be in [1, 8]")
        if atm.engine != "spectral" or atm._boiling or atm._lgs_mag is not None:
            raise ValueError("frame_loop needs the spectral engine without boiling or LGS")
        if not dt > 0:
            raise ValueError("dt must be positive")
        if int(steps) < 1:
            raise ValueError("steps must be >= 1")
        self.atm, self.dt, self.steps = atm, float(dt), int(steps)
        spec = atm._spec
        self._spec = spec
        self._P = spec.P
        self.times = np.empty(self.steps)
        t = 0.0
        for i in range(self.steps):  # the reference's clock: repeated float additions
            self.times[i] = t
            t += self.dt
        self._sx = np.ascontiguousarray(atm._vx[None, :] * self.times[:, None])
        self._sy = np.ascontiguousarray(atm._vy[None, :] * self.times[:, None])
        self._scale = atm._scale(wavelength)
        self._spectra = spec.spectra.clone()
        self._sh = spec.sh_coef.clone()
        dev = spec.grid.device
        self.out = torch.empty((self.steps, atm.n, atm.n), dtype=torch.float32, device=dev)
        self._work = [spec.grid.work]
        self._side = []
        self.graph = None
        self.capture(branches)

    def capture(self, branches: int) -> None:
        """(Re)capture the graph with ``branches`` branches: chunk c goes to
        stream c % branches with its own workspace, so one chunk's
        latency-bound launches overlap another's."""
        torch = torch_module()
        branches = int(branches)
        if not 1 <= branches <= 8:
            raise ValueError("branches must be in [1, 8]")
        dev = self._spec.grid.device
        self.branches = branches
        while len(self._work) < branches:
            self._work.append(torch.empty(self._spec.grid.work_bytes, dtype=torch.uint8,
                                          device=dev))
        while len(self._side) < branches - 1:
            self._side.append(torch.cuda.Stream(dev))
        self.graph = None
        self._render_body()                      # first launches outside the capture
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
            self._render_body()
        torch.cuda.synchronize(dev)

    def _render_body(self) -> None:
        torch = torch_module()
        spec, atm, k = self._spec, self.atm, self.atm.frames_chunk
        main = torch.cuda.current_stream()
        side = self._side[:self.branches - 1]
        streams = [main] + side
        for sd in side:
            sd.wait_stream(main)
        for c, c0 in enumerate(range(0, self.steps, k)):
            m = min(k, self.steps - c0)
            b = c % self.branches
            _lib.call("pt_frames", spec.grid.handle, spec.L, dptr(self._spectra),
                      dptr(self._sh) if self._P else None, m,
                      _lib.as_dptr(self._sx[c0:c0 + m]), _lib.as_dptr(self._sy[c0:c0 + m]), 0,
                      int(atm.margin_pix), int(atm.n), float(self._scale), dptr(self.out[c0:c0 + m]),
                      dptr(self._work[b]), spec.grid.work_bytes, streams[b].cuda_stream)
        for sd in side:
            main.wait_stream(sd)

    def render(self, t0: float):
        """Frames at ``t0 + times`` into :attr:`out` (returned), ``(steps, n, n)``."""
        atm, spec = self.atm, self._spec
        sx0 = np.ascontiguousarray(atm._vx * float(t0), dtype=np.float64)
        sy0 = np.ascontiguousarray(atm._vy * float(t0), dtype=np.float64)
        if not atm._wrap_warned:
            atm._check_wrap(sx0[None, :] + self._sx[-1:], sy0[None, :] + self._sy[-1:])
        _lib.call("pt_layers_translate", spec.grid.handle, spec.L, dptr(spec.spectra),
                  dptr(spec.sh_coef) if self._P else None, _lib.as_dptr(sx0), _lib.as_dptr(sy0),
                  dptr(self._spectra), dptr(self._sh) if self._P else None, stream_handle())
        self.graph.replay()
        return self.out
