"""Benchmark: 9-layer 512^2 OPD frames/s (spectral frozen flow) and Monte-Carlo
screens/s on the GB300, with the reference's CPU path timed beside it.

Workload (one step): ``Atmosphere`` with 9 layers at h = [0, 0.5, 1, 2, 4, 8,
12, 16, 20] km, Cn2 fractions [0.52, 0.10, 0.07, 0.06, 0.05, 0.06, 0.06, 0.05,
0.03], winds U[5, 30] m/s with seeded directions, n = 512, D = 8 m,
r0 = 0.157 m, L0 = 25 m, zenith 30 deg, 3 subharmonic levels, dt = 1 ms:
2000 frames rendered into HBM. Secondary: ``Atmosphere.sample(64)`` at 512^2
(MC screens/s), the metric's tensor-core form of the 512^2 transform beside
the FP32 FFT (``dft_512_tc_vs_fp32``), config 1 generate, config 3
extrusion, config 4 differentiable readout and config 5 ragged ensembles.
Synthetic seeded inputs throughout.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs under torchrun: each rank renders its own, disjoint time window
(replicas, weak scaling); rank 0 prints the JSON line with the max time over
ranks. ``--impl reference`` times the reference's own CPU path (the float32
NumPy/SciPy port in ``oracle/baseline.py``) on the host cores.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HEIGHTS = [0, 500, 1000, 2000, 4000, 8000, 12000, 16000, 20000]
FRACTIONS = [0.52, 0.10, 0.07, 0.06, 0.05, 0.06, 0.06, 0.05, 0.03]
N_PIX, DIAM, R0, L0, ZENITH, LEVELS, DT = 512, 8.0, 0.157, 25.0, 30.0, 3, 1e-3
FRAMES_PER_STEP = 2000
MC_BATCH = 64
WORKLOAD = ("spectral frozen flow: 9 layers, 512^2 pupil, D=8 m, r0=0.157 m, L0=25 m, "
            "z=30 deg, 3 subharmonic levels, dt=1 ms, 2000 frames per step")
METRIC = "9-layer 512^2 OPD frames/s"


def layer_table(seed: int = 2024):
    rng = np.random.default_rng(seed)
    speeds = rng.uniform(5.0, 30.0, 9)
    dirs = rng.uniform(0.0, 360.0, 9)
    return list(zip(HEIGHTS, FRACTIONS, speeds, dirs))


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def captured_traffic(kernel: str, frames_per_launch: float):
    """DRAM bytes per launch of ``kernel`` from the committed ncu capture
    (``profiles/dram_traffic.json``), scaled to ``frames_per_launch``; the
    kernels' traffic grows in proportion to the frames a launch renders."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    b = d.get("bytes_per_launch", {}).get(kernel)
    if b is None:
        return None
    return float(b) * frames_per_launch / float(d["frames_per_launch"])


class Clocks:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"pt_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _reference_cpu(ReferenceCPU):
    """The bench workload on the reference's CPU path, and the cores it uses."""
    tab = layer_table()
    cos_z = np.cos(np.deg2rad(ZENITH))
    frac = np.array(FRACTIONS) / np.sum(FRACTIONS)
    r0_los = R0 * cos_z ** 0.6
    r0s = [r0_los * f ** (-0.6) for f in frac]
    vx = [v * np.cos(np.deg2rad(d)) for _, _, v, d in tab]
    vy = [v * np.sin(np.deg2rad(d)) for _, _, v, d in tab]
    alt = [h / cos_z for h, *_ in tab]
    ref = ReferenceCPU(N_PIX, N_PIX, DIAM / N_PIX, r0s, [L0] * 9, LEVELS, vx, vy, alt, 0,
                       workers=-1)
    return ref, len(os.sched_getaffinity(0))


def cpu_reference(frames: int, mc_count: int, budget_s: float = 12.0):
    """Time the reference CPU path (float32 NumPy/SciPy port) on a bounded sample."""
    import warnings

    from oracle.baseline import ReferenceCPU

    warnings.simplefilter("ignore")
    tab = layer_table()
    cos_z = np.cos(np.deg2rad(ZENITH))
    frac = np.array(FRACTIONS) / np.sum(FRACTIONS)
    r0_los = R0 * cos_z ** 0.6
    r0s = [r0_los * f ** (-0.6) for f in frac]
    vx = [v * np.cos(np.deg2rad(d)) for _, _, v, d in tab]
    vy = [v * np.sin(np.deg2rad(d)) for _, _, v, d in tab]
    alt = [h / cos_z for h, *_ in tab]
    cores = len(os.sched_getaffinity(0))
    ref = ReferenceCPU(N_PIX, N_PIX, DIAM / N_PIX, r0s, [L0] * 9, LEVELS, vx, vy, alt, 0,
                       workers=-1)
    for k in range(3):
        ref.frame(k * DT)
    t0 = time.perf_counter()
    done = 0
    while done < frames and time.perf_counter() - t0 < budget_s:
        ref.frame(done * DT)
        done += 1
    fps = done / (time.perf_counter() - t0)
    rng = np.random.default_rng(0)
    ref.sample(mc_count, rng)
    t0 = time.perf_counter()
    drawn = 0
    while drawn < 4 * mc_count and time.perf_counter() - t0 < budget_s / 2:
        ref.sample(mc_count, rng)
        drawn += mc_count
    sps = drawn / (time.perf_counter() - t0)
    return fps, sps, cores, done, drawn


def bench_generate(torch, G):
    """PhaseScreen.generate(64) at 256^2 (D = 8 m, r0 = 0.15, L0 = 25, 3 levels): screens/s."""
    gen = G.PhaseScreen(n=256, pixel_scale=8.0 / 256, r0=0.15, L0=25.0, subharmonics=3, seed=5)
    out = torch.empty((64, 256, 256), dtype=torch.float32, device="cuda")
    for _ in range(3):
        gen._generate_into(out, 64, 0, 256, 1.0, False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 50
    e0.record()
    for _ in range(reps):
        gen._generate_into(out, 64, 0, 256, 1.0, False)
    e1.record()
    torch.cuda.synchronize()
    return reps * 64 / (e0.elapsed_time(e1) / 1000.0)


def _dft_calls(torch, n: int, batch: int):
    """The two inverse 2-D DFT forms over the same (batch, n, n) complex
    buffers: the tensor-core four-step (pt_ifft2_tc) and the FP32 register FFT
    (pt_ifft2)."""
    from pyturb_gb300 import _lib
    from pyturb_gb300.backend import stream_handle
    from pyturb_gb300.fourier import Grid

    x = torch.randn((batch, n, n, 2), device="cuda")
    y = torch.empty_like(x)
    g = Grid(n, 0.01, np.zeros((0, 3)))

    def tc():
        _lib.call("pt_ifft2_tc", n, x.data_ptr(), y.data_ptr(), batch, stream_handle())

    def fp32():
        _lib.call("pt_ifft2", g.handle, x.data_ptr(), y.data_ptr(), batch, g.work.data_ptr(),
                  g.work_bytes, stream_handle())

    return x, y, {"tc_fp16x2": tc, "fp32_fft": fp32}


def bench_tc_dft(torch, batch: int = 96, reps: int = 20) -> dict:
    """The transform under every 512^2 frame and Monte-Carlo screen, in its two
    forms: the inverse 2-D DFT of `batch` complex 512^2 images (192 MB in,
    192 MB out, above the L2) as split-bf16 tensor-core four-step DFTs, and as
    the FP32 register FFT; transforms/s and relative L2 against float64."""
    n = 512
    x, y, forms = _dft_calls(torch, n, batch)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res = {"workload": f"inverse 2-D DFT of {batch} complex {n}^2 images per call "
                       "(row pass + column pass), inputs above L2"}
    # accuracy on a coloured spectrum (steep power law, like the screens')
    rng = np.random.default_rng(3)
    f = np.fft.fftfreq(n)
    amp = (f[:, None] ** 2 + f[None, :] ** 2 + 1e-4) ** (-11.0 / 12.0)
    z = (rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))) * amp
    exact = np.fft.ifft2(z) * (n * n)
    x[:2].copy_(torch.from_numpy(np.stack([z.real, z.imag], -1).astype(np.float32)))
    for name, fn in forms.items():
        fn()
        torch.cuda.synchronize()
        o = y[:2].double().cpu().numpy()
        err = float(np.linalg.norm(o[..., 0] + 1j * o[..., 1] - exact) / np.linalg.norm(exact))
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1000.0 / reps
        res[name] = {"transforms_per_s": batch / sec, "us_per_transform": sec / batch * 1e6,
                     "two_pass_gbs": batch * n * n * 8 * 4 / sec / 1e9,
                     "rel_l2_vs_fp64": err}
    res["tc_over_fp32"] = res["tc_fp16x2"]["transforms_per_s"] / res["fp32_fft"]["transforms_per_s"]
    # both pipelines spend one 512^2 complex transform per two real screens or
    # frames, so the transform rate bounds the screens/s any form of them reaches
    res["tc_form_bound_screens_or_frames_per_s"] = 2.0 * res["tc_fp16x2"]["transforms_per_s"]
    res["note"] = ("tc_fp16x2 = 512 = 32 x 16 four-step DFT: per pass, the (line, n2) x 32-point "
                   "and (line, k1) x 16-point DFT block matrices as tcgen05 kind::f16 products "
                   "of two-term fp16 splits of power-of-two scaled lines (three products, fp32 "
                   "accumulation in tensor memory), twiddles in registers; persistent "
                   "256-thread CTAs, two per SM, the next 8-line group prefetched with "
                   "16-byte cp.async (column groups staged transposed). "
                   "fp32_fft = the register FFT under generate / sample / frames, where "
                   "it is fused with the noise, recurrence and subharmonic work. The tc "
                   "bound counts the transform alone (no spectrum fill, no pair "
                   "extraction): a whole tc-form pipeline is slower than that")
    return res


def extrude_accuracy(torch, G, ext, r0s, steps: int = 512, screens: int = 3) -> dict:
    """Relative L2 error of each extrusion form against a float64 recursion
    with the same operator and injected noise: `screens` ring screens of the
    atmosphere's geometry (layers 0, 4, 8), `steps` row steps, compared over
    the last 128 rows. The float64 operator is the device build's own."""
    from pyturb_gb300.backend import NoiseStream
    from pyturb_gb300.covariance import AnchorTables, build_operator
    from pyturb_gb300.extrude import RingExtruder

    W, cap, sparse, dx = ext.width, ext.capacity, ext.sparse, ext.dx
    layers = [0, 4, 8][:screens]
    depth = max([2] + [d for d, _ in sparse])
    bscale = [r0s[i] ** (-5.0 / 6.0) for i in layers]
    seed = [ext._ring.buf[i, :depth].clone() for i in layers]  # ring rows 0 .. depth - 1
    op = build_operator(W, 2, dx, L0, sparse, b_factor="eigh", want_float64=True,
                        want_lo=bool(sparse))
    a, b = op.host()  # the float64 recursion
    R = [np.concatenate([x.double().cpu().numpy(), np.empty((steps, W))]) for x in seed]
    st = [NoiseStream(700 + q, np.random.default_rng) for q in range(len(layers))]
    for t in range(depth, depth + steps):
        Z = np.stack([np.concatenate([r[t - 2:t].ravel(), [r[t - d, c] for d, c in sparse]])
                      for r in R], axis=1)
        beta = np.stack([st[q].draw((W,)) * bscale[q] for q in range(len(layers))], axis=1)
        new = a @ Z + b @ beta
        for q, r in enumerate(R):
            r[t] = new[:, q]
    opi = build_operator(W, 2, dx, L0, sparse, b_factor="eigh", increments=True)
    out = {}
    sp_modes = 64 if sparse else 32
    for name, form, anchor in (("fp32", "fp32", AnchorTables([op], sp_modes)),
                               ("fp32_unanchored", "fp32", None), ("bf16x2", "bf16x2", None),
                               ("bf16x3", "bf16x3", None)):
        ring = RingExtruder(W, 2, cap, [], [0] * len(layers), bscale,
                            [NoiseStream(700 + q, np.random.default_rng) for q in range(len(layers))],
                            device_operator=opi.M if form == "bf16x3" else op.M, form=form,
                            sparse=sparse, anchor=anchor, increments=form == "bf16x3",
                            operator_lo=op.Mlo if anchor is not None and sparse else None)
        for q in range(len(layers)):
            ring.seed_rows(q, seed[q])
        ring.extrude(np.full(len(layers), steps, dtype=np.int32))
        torch.cuda.synchronize()
        top = int(ring.top[0])
        phys = [(top - k - 1) % cap for k in range(128)][::-1]
        got = ring.buf[:, phys].double().cpu().numpy()
        want = np.stack([r[-128:] for r in R])
        out[name] = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        del ring
    return out


def bench_extrude(torch, G, steps: int = 4096):
    """Assemat-Wilson extrusion at n = 1024 with the configured stencil (2 full
    rows + 2 sparse columns), 9 layers x 16 realisations = 144 ring screens,
    4096 row steps (one [A | B] GEMM per row step: M = W, N = 144,
    K = 3 W + 18), in each product form; the rows-only stencil beside it; and
    the fused 9-layer bilinear readout of one realisation at 1024^2."""
    from pyturb_gb300 import _lib
    from pyturb_gb300.backend import NoiseStream, stream_handle
    from pyturb_gb300.covariance import build_operator
    from pyturb_gb300.extrude import RingExtruder

    tab = layer_table()
    n = 1024
    cos_z = np.cos(np.deg2rad(ZENITH))
    frac = np.array(FRACTIONS) / np.sum(FRACTIONS)
    r0s = [R0 * cos_z ** 0.6 * f ** (-0.6) for f in frac]
    winds = [(v * np.cos(np.deg2rad(d)), v * np.sin(np.deg2rad(d))) for _, _, v, d in tab]
    R = 16
    S = 9 * R
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ones = np.ones(S, dtype=np.int32)
    out = {}
    for columns in (2, 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ext = G.ExtrudedAtmosphere(n=n, pixel_scale=DIAM / n, layer_r0=r0s, layer_L0=[L0] * 9,
                                   layer_wind=winds,
                                   layer_altitude_los=[h / cos_z for h in HEIGHTS],
                                   interp="linear", seeds=list(range(9)),
                                   stencil_columns=columns)
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        W, cap, sparse = ext.width, ext.capacity, ext.sparse
        K = 3 * W + len(sparse)
        flops = 2.0 * W * K * S
        if columns == 2:
            accuracy = extrude_accuracy(torch, G, ext, r0s)
        res = {"stencil": f"2 full rows + {columns} sparse columns ({len(sparse)} points)",
               "W": W, "K": K, "host_setup_s": setup_s, "forms": {}}
        # bf16x3 runs the increment form of the same operator
        inc = build_operator(W, 2, DIAM / n, L0, sparse, increments=True).M
        variants = (("fp32", "fp32", ext._ring.anchor), ("fp32_unanchored", "fp32", None),
                    ("bf16x2", "bf16x2", None), ("bf16x3", "bf16x3", None))
        for name, form, anchor in variants:
            ring = RingExtruder(W, 2, cap, [], [0] * S, [r ** (-5.0 / 6.0) for r in r0s] * R,
                                [NoiseStream(100 + s, None) for s in range(S)],
                                device_operator=inc if form == "bf16x3" else ext._ring.M,
                                form=form, sparse=sparse, anchor=anchor,
                                operator_lo=ext._ring.M_lo if anchor is not None else None,
                                increments=form == "bf16x3")
            for s in range(S):  # every realisation starts from layer (s % 9)'s seeded rows
                ring.buf[s].copy_(ext._ring.buf[s % 9])
                ring.top[s] = ext._ring.top[s % 9]
            for _ in range(3):
                ring.extrude(ones)
            torch.cuda.synchronize()
            e0.record()
            ring.extrude(steps * ones)
            e1.record()
            torch.cuda.synchronize()
            st = e0.elapsed_time(e1) / 1000.0 / steps
            # per-kernel event timings in a separate pass (the events cost time)
            _lib.prof_report()
            _lib.prof_enable(True)
            ring.extrude(256 * ones)
            torch.cuda.synchronize()
            prof = _lib.prof_report()
            _lib.prof_enable(False)
            g = prof.get("k_tc_gemm" if form != "fp32" else "k_extrude_gemm", (1, float("nan")))
            gemm_s = g[1] / g[0] / 1e3
            products = {"fp32": 1, "bf16x2": 3, "bf16x3": 6}[form]
            res["forms"][name] = {
                "row_steps_per_s": 1.0 / st, "effective_tflops": flops / st / 1e12,
                "gemm_us": gemm_s * 1e6, "gemm_tflops_issued": products * flops / gemm_s / 1e12,
                "kernel_us_per_step": {k: round(v[1] / 256 * 1e3, 2) for k, v in prof.items()},
                "rel_l2_vs_fp64_512_steps": accuracy[name] if columns == 2 else None}
            del ring
        for f32 in (res["forms"]["fp32"], res["forms"]["fp32_unanchored"]):
            f32["gemm_kernel_frac_of_fp32_nominal"] = f32["gemm_tflops_issued"] / 80.5
        if columns == 2:
            # readout: the 9 layers of one realisation, bilinear, at 1024^2
            o = torch.empty((n, n), dtype=torch.float32, device="cuda")
            ext.set_time(0.01)
            params = ext.readout_params()
            for _ in range(3):
                ext.integrate(out=o)
            torch.cuda.synchronize()
            e0.record()
            reps = 50
            for _ in range(reps):
                _lib.call("pt_readout", n, W, cap, 0, 9, params, ext._buf.data_ptr(), 1.0,
                          o.data_ptr(), stream_handle())
            e1.record()
            torch.cuda.synchronize()
            ro_s = e0.elapsed_time(e1) / 1000.0 / reps
            res["readout_frames_per_s"] = 1.0 / ro_s
            res["readout_gbs_out"] = n * n * 4 / ro_s / 1e9
            # one bilinear tap set (2 x 2 samples) per pixel and layer; the 9
            # rings (W x cap floats each) stay L2-resident across frames, so
            # DRAM sees little beyond the frame written
            res["readout_pixel_layers_per_s"] = 9 * n * n / ro_s
            res["readout_bytes_per_frame_algorithmic"] = n * n * 4 + 9 * n * n * 4
        out["configured" if columns == 2 else "rows_only"] = res
        del ext
    cfg = out["configured"]
    return {"workload": f"n=1024, 9 layers x {R} realisations ({S} screens), "
                        f"W={cfg['W']}, stencil {cfg['stencil']}, {steps} row steps timed per "
                        "form; readout bilinear 9 layers",
            "row_steps_per_s": cfg["forms"]["fp32"]["row_steps_per_s"],
            "note": "fp32 = register-tiled split-K SIMT FP32 GEMM plus the 32-mode double-float "
                    "low-order anchor (the default, parity form); fp32_unanchored = the same "
                    "without it; bf16x2/x3 = split-bf16 tcgen05 products (bf16x3 on the "
                    "increment-form operator). FP32 nominal 80.5 TFLOP/s = 152 SMs x 128 lanes x 2 x 2.07 GHz; "
                    "operator built in FP64 on the GPU (host_setup_s includes seeding the 9 rings)",
            **out}


def bench_diff(torch, G, iters: int = 3):
    """Differentiable readout: 9 layers of 768^2 screens (generate-coloured),
    8 directions in a 60 arcsec disc + 1 LGS at 90 km, 512^2 pupil, batch 32,
    64 frames at 1 ms; MSE to a target rendered with perturbed Cn2 weights and
    winds; one Adam step on 9 weights + 18 wind components per iteration
    (forward, loss, backward wrt screens, weights and winds, update)."""
    from pyturb_gb300 import _lib
    from pyturb_gb300.diff import DifferentiableReadout

    B, L, S, n, T = 32, 9, 768, 512, 64
    dx = DIAM / n
    rng = np.random.default_rng(77)
    rad = np.deg2rad(60.0 / 3600.0) * np.sqrt(rng.uniform(0, 1, 8))
    ang = rng.uniform(0, 2 * np.pi, 8)
    dirs = np.concatenate([np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1), [[0.0, 0.0]]])
    ro = DifferentiableReadout(n, S, dx, HEIGHTS, dirs, np.arange(T) * DT,
                               source_altitudes=[None] * 8 + [90e3])
    gen = G.PhaseScreen(n=S, pixel_scale=dx, r0=R0, L0=L0, subharmonics=LEVELS, seed=9)
    screens = gen.generate(B * L).reshape(B, L, S, S).contiguous()
    tab = layer_table()
    v_true = torch.tensor([[v * np.cos(np.deg2rad(d)), v * np.sin(np.deg2rad(d))]
                           for _, _, v, d in tab], dtype=torch.float64, device="cuda")
    w_true = torch.tensor(np.sqrt(FRACTIONS), dtype=torch.float32, device="cuda")
    with torch.no_grad():
        target = ro(screens, w_true * torch.tensor(rng.uniform(0.8, 1.2, L), dtype=torch.float32,
                                                    device="cuda"),
                    v_true + torch.tensor(rng.normal(0, 1.0, (L, 2)), device="cuda"))
    screens.requires_grad_(True)
    w = w_true.clone().requires_grad_(True)
    v = v_true.clone().requires_grad_(True)
    opt = torch.optim.Adam([w, v], lr=0.01)

    def step():
        opt.zero_grad(set_to_none=True)
        screens.grad = None
        loss = torch.nn.functional.mse_loss(ro(screens, w, v), target)
        loss.backward()
        opt.step()
        return loss

    chunk = 8

    def step_ckpt():
        opt.zero_grad(set_to_none=True)
        screens.grad = None
        loss = ro.mse(screens, w, v, target, frames_per_chunk=chunk)
        loss.backward()
        opt.step()
        return loss

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    forms = {}
    for name, fn in (("checkpointed", step_ckpt), ("materialised", step)):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        e0.record()
        for _ in range(iters):
            loss = fn()
        e1.record()
        torch.cuda.synchronize()
        forms[name] = {"iter_ms": e0.elapsed_time(e1) / iters,
                       "peak_gb": torch.cuda.max_memory_allocated() / 1e9,
                       "peak_above_inputs_gb": (torch.cuda.max_memory_allocated() - base) / 1e9,
                       "loss": float(loss.detach())}
    forms["checkpointed"]["frames_per_chunk"] = chunk
    it_s = forms["materialised"]["iter_ms"] / 1000.0
    # per-kernel event timings in a separate iteration (the events cost time)
    _lib.prof_report()
    _lib.prof_enable(True)
    loss = step()
    torch.cuda.synchronize()
    prof = _lib.prof_report()
    _lib.prof_enable(False)
    units = B * T  # (batch, frame) pairs per iteration
    fwd_b = L * S * S * 4 + 9 * n * n * 4  # algorithmic bytes per (batch, frame), forward
    k = {name: v[1] / v[0] / 1000.0 for name, v in prof.items()}
    fwd_s = k.get("k_lr_forward", float("nan"))
    return {"workload": "9 layers 768^2 x batch 32, 8 NGS dirs in 60\" + 1 LGS at 90 km, "
                        "pupil 512^2, 64 frames, MSE + Adam on 9 weights + 18 winds",
            "iter_ms": it_s * 1e3, "frames_per_s": units / it_s,
            "kernel_ms": {name: v * 1e3 for name, v in k.items()},
            "forward_gbs_algorithmic": units * fwd_b / fwd_s / 1e9,
            "loss": float(loss.detach()),
            "forms": forms,
            "note": "materialised = torch MSE of the full (32, 64, 9, 512, 512) frame tensor; "
                    "checkpointed = readout_mse: loss only in the forward, frames recomputed "
                    "8 time steps at a time in the backward (screens are the checkpoint); "
                    "peak_gb = torch's peak allocation during the timed iterations (the "
                    "19.3 GB target and the 0.68 GB screens included)"}


def bench_ragged(torch, reps: int = 5):
    """Ragged Monte-Carlo ensemble: 4096 screens with n drawn from {128, 256,
    384, 512, 1024} (weights 4:4:2:2:1), L0 from {10, 25, 50} m, r0 ~ U[0.08,
    0.25] m, dx = 1/64 m, 3 subharmonic levels, seeded; one pt_generate_scaled
    call per (n, L0) group per ensemble."""
    from pyturb_gb300 import _lib
    from pyturb_gb300.ragged import RaggedEnsemble

    rng = np.random.default_rng(55)
    S = 4096
    sizes = rng.choice([128, 256, 384, 512, 1024], size=S, p=np.array([4, 4, 2, 2, 1]) / 13.0)
    L0s = rng.choice([10.0, 25.0, 50.0], size=S)
    r0s = rng.uniform(0.08, 0.25, S)
    ens = RaggedEnsemble(sizes, r0s, L0s, pixel_scale=1.0 / 64, subharmonics=3, seed=55,
                         autotune=True)  # tuned at construction, outside the timing
    for _ in range(2):
        ens.generate()
    torch.cuda.synchronize()
    c0 = _lib.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        ens.generate()
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1000.0 / reps
    out_bytes = 4.0 * float(np.sum(sizes.astype(np.float64) ** 2))
    hbm, _, _ = peaks()
    return {"workload": "4096 screens, n in {128,256,384,512,1024} w 4:4:2:2:1, L0 in "
                        "{10,25,50} m, r0 ~ U[0.08,0.25] m, dx 1/64 m, 3 subharmonic levels",
            "screens_per_s": S / sec, "ms_per_ensemble": sec * 1e3,
            "output_gb": out_bytes / 1e9, "output_gbs": out_bytes / sec / 1e9,
            "output_frac_of_hbm": out_bytes / sec / 1e9 / hbm,
            "groups": ens.n_groups, "launches_per_ensemble": (_lib.launch_count() - c0) // reps}


def bench_config(world: int) -> dict:
    """The workload description both arms print (same keys, same values)."""
    return {"workload": WORKLOAD, "frames_per_step": FRAMES_PER_STEP,
            "l2": "flushed between steps by a 256 MB write outside the step events",
            "parallelism": f"replicas x{world} (disjoint time windows)",
            "frame_loop": "CUDA graph of the 2000-frame loop, replayed per window after "
                          "one pt_layers_translate launch (Atmosphere.frame_loop)",
            "noise": "in-kernel Philox4x32-10"}


REF_FRAMES_PER_STEP = 100  # frames of the 2000-frame window timed per reference step
REF_MC_PER_STEP = 64       # Monte-Carlo screens timed per reference step


def run_reference(args, rank: int) -> None:
    """The reference's CPU path on the host cores: each step renders the first
    100 frames of its 2000-frame window and draws 64 MC screens, and is timed
    as a whole (ms_per_step is the measured time of exactly that work)."""
    if rank != 0:
        return
    import warnings

    from oracle.baseline import ReferenceCPU

    warnings.simplefilter("ignore")
    ref, cores = _reference_cpu(ReferenceCPU)
    rng = np.random.default_rng(0)
    frame_s, mc_s = [], []
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for k in range(REF_FRAMES_PER_STEP):
            ref.frame((s * FRAMES_PER_STEP + k) * DT)
        t1 = time.perf_counter()
        ref.sample(REF_MC_PER_STEP, rng)
        t2 = time.perf_counter()
        if s >= args.warmup:
            frame_s.append(t1 - t0)
            mc_s.append(t2 - t1)
    fps = REF_FRAMES_PER_STEP * len(frame_s) / sum(frame_s)
    sps = REF_MC_PER_STEP * len(mc_s) / sum(mc_s)
    line = {
        "impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * (sum(frame_s) + sum(mc_s)) / len(frame_s),
        "frames_per_step_timed": REF_FRAMES_PER_STEP, "mc_screens_per_step_timed": REF_MC_PER_STEP,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": bench_config(1),
        "mc_screens_per_s": sps,
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": f"per step {REF_FRAMES_PER_STEP} frames of the 2000-frame "
                                   f"window and {REF_MC_PER_STEP} MC screens, all timed; "
                                   "float32 NumPy/SciPy port of Atmosphere._integrate / "
                                   "PhaseScreen.generate (oracle/baseline.py), scipy FFT "
                                   "workers = all cores"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_case(args) -> None:
    """One small, named workload for profiling a kernel family under ncu (no
    JSON line): ``generate`` (``--n``, ``--count``, ``--calls``),
    ``extrude`` (``--width``, ``--screens``, ``--case-steps``, ``--form``) or
    ``dft`` (512^2 x ``--count`` inverse DFTs, ``--calls``; ``--form`` fp32 for
    the FFT, else the tensor-core form) or ``readout`` (the 9-layer bilinear
    extruder readout at ``--n``, ``--calls`` frames)."""
    import torch

    import pyturb_gb300 as G
    from pyturb_gb300 import _lib
    from pyturb_gb300.backend import NoiseStream, cuda_device
    from pyturb_gb300.covariance import AnchorTables, build_operator
    from pyturb_gb300.extrude import RingExtruder

    torch.cuda.set_device(0)
    if args.case == "dft":
        _x, _y, forms = _dft_calls(torch, 512, args.count)
        fn = forms["tc_fp16x2" if args.form != "fp32" else "fp32_fft"]
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.calls):
            fn()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / max(1, args.calls)
        print(f"dft 512^2 x {args.count} form={args.form}: {dt * 1e6:.1f} us per call")
        return
    if args.case == "readout":
        # the 9-layer bilinear readout of one realisation at n = --n (1024 in the bench)
        from pyturb_gb300.backend import stream_handle

        n = args.n
        tab = layer_table()
        cos_z = np.cos(np.deg2rad(ZENITH))
        frac = np.array(FRACTIONS) / np.sum(FRACTIONS)
        r0s = [R0 * cos_z ** 0.6 * f ** (-0.6) for f in frac]
        winds = [(v * np.cos(np.deg2rad(d)), v * np.sin(np.deg2rad(d))) for _, _, v, d in tab]
        ext = G.ExtrudedAtmosphere(n=n, pixel_scale=DIAM / n, layer_r0=r0s, layer_L0=[L0] * 9,
                                   layer_wind=winds,
                                   layer_altitude_los=[h / cos_z for h in HEIGHTS],
                                   interp="linear", seeds=list(range(9)))
        o = torch.empty((n, n), dtype=torch.float32, device="cuda")
        ext.set_time(0.01)
        params = ext.readout_params()
        ext.integrate(out=o)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.calls):
            _lib.call("pt_readout", n, ext.width, ext.capacity, 0, 9, params,
                      ext._buf.data_ptr(), 1.0, o.data_ptr(), stream_handle())
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / max(1, args.calls)
        print(f"readout n={n} 9 layers: {dt * 1e6:.1f} us per frame")
        return
    if args.case == "generate":
        g = G.PhaseScreen(n=args.n, pixel_scale=8.0 / args.n, r0=0.15, L0=25.0,
                          subharmonics=3, seed=1)
        g.generate(args.count)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.calls):
            g.generate(args.count)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / max(1, args.calls)
        print(f"generate n={args.n} count={args.count}: {dt * 1e6:.1f} us per call")
        return
    W, m, S = args.width, 2, args.screens
    fp32, inc = args.form == "fp32", args.form == "bf16x3"
    op = build_operator(W, m, 8.0 / 1024, 25.0, want_float64=fp32, increments=inc)
    ring = RingExtruder(W, m, args.case_steps + m + 8, [], [0] * S, [1.0] * S,
                        [NoiseStream(100 + s, None) for s in range(S)], form=args.form,
                        device_operator=op.M, anchor=AnchorTables([op]) if fp32 else None,
                        increments=inc)
    for s in range(S):
        ring.seed_rows(s, torch.zeros((m, W), device=cuda_device()))
    ring.extrude(np.ones(S, dtype=np.int32))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ring.extrude(np.full(S, args.case_steps - 1, dtype=np.int32))
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / max(1, args.case_steps - 1)
    print(f"extrude form={args.form} W={W} screens={S}: {dt * 1e6:.1f} us per row step")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extrude", action="store_true")
    ap.add_argument("--no-diff", action="store_true")
    ap.add_argument("--case", choices=["generate", "extrude", "dft", "readout"], default=None,
                    help="run one small named workload for profiling and exit")
    ap.add_argument("--n", type=int, default=384)
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--calls", type=int, default=4)
    ap.add_argument("--width", type=int, default=1449)
    ap.add_argument("--screens", type=int, default=144)
    ap.add_argument("--case-steps", type=int, default=16)
    ap.add_argument("--form", default="fp32", choices=["fp32", "bf16x2", "bf16x3"])
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)

    import warnings

    import pyturb_gb300 as G
    from pyturb_gb300 import _lib, replicas

    warnings.simplefilter("ignore")
    dev = torch.device("cuda", torch.cuda.current_device())
    layers = [G.Layer(h, f, v, d, L0) for h, f, v, d in layer_table()]
    atm = G.Atmosphere(layers, r0=R0, zenith_angle=ZENITH, diameter=DIAM, n=N_PIX,
                       subharmonics=LEVELS, seed=replicas.rank_seed(1000, rank, world),
                       frames_chunk=64)
    out = torch.empty((FRAMES_PER_STEP, N_PIX, N_PIX), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    # each rank renders its own, disjoint time window
    def step_times(s: int) -> np.ndarray:
        return replicas.time_window(rank, s, FRAMES_PER_STEP, DT)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- headline: the CUDA-graph frame loop (the chunked frame launches
    # captured once; per 2000-frame window one pt_layers_translate launch and
    # one replay). Every frame of every window is rendered again.
    stream = torch.cuda.current_stream()
    c0 = _lib.launch_count()
    loop = atm.frame_loop(DT, FRAMES_PER_STEP)
    kernels_per_replay = (_lib.launch_count() - c0) // 2  # warm-up call + captured call
    c1 = _lib.launch_count()
    loop.render(0.0)
    translate_kernels = _lib.launch_count() - c1
    for s in range(args.warmup):
        loop.render(float(step_times(s)[0]))
    barrier()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    barrier()
    wall0 = time.perf_counter()
    events = []
    for s in range(args.steps):
        flush.fill_(s & 0xFF)  # evict L2 between steps (outside the step's events)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        loop.render(float(step_times(args.warmup + s)[0]))
        e1.record(stream)
        events.append((e0, e1))
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    launches = args.steps * (kernels_per_replay + translate_kernels)
    step_ms = [a.elapsed_time(b) for a, b in events]
    total_ms = replicas.max_over_ranks(float(sum(step_ms)), dist, dev)
    frames_total = world * args.steps * FRAMES_PER_STEP
    value = frames_total / (total_ms / 1000.0)
    del loop

    # ---- the same windows launched chunk by chunk (no graph); then a second
    # pass with every kernel timed by CUDA events on its stream: the
    # per-kernel figures of the roofline (the graph replays exactly these
    # kernels; the events are kept out of the timed pass)
    for s in range(args.warmup):
        atm.render(step_times(s), out=out)
    barrier()
    devents = []
    for s in range(args.steps):
        flush.fill_(s & 0xFF)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        atm.render(step_times(args.warmup + s), out=out)
        e1.record(stream)
        devents.append((e0, e1))
    barrier()
    _lib.prof_report()  # clear
    _lib.prof_enable(True)
    for s in range(args.steps):
        flush.fill_(s & 0xFF)
        atm.render(step_times(args.warmup + s), out=out)
    barrier()
    prof = _lib.prof_report()
    _lib.prof_enable(False)
    direct_ms = replicas.max_over_ranks(float(sum(a.elapsed_time(b) for a, b in devents)), dist,
                                        dev)
    direct = {"frames_per_s": frames_total / (direct_ms / 1000.0),
              "ms_per_step": direct_ms / args.steps,
              "path": "Atmosphere.render(times) per 2000-frame window: 32 chunks of "
                      "pt_frames launched from the host"}

    # ---- end to end through the public API: every frame delivered to pinned host memory
    host = torch.empty((FRAMES_PER_STEP, N_PIX, N_PIX), dtype=torch.float32, pin_memory=True)
    e2e_ms = []
    for s in range(3):
        atm.reset()
        barrier()
        t0 = time.perf_counter()
        atm.frames_host(dt=DT, steps=FRAMES_PER_STEP, out=host)
        torch.cuda.synchronize()
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    e2e_step = replicas.max_over_ranks(min(e2e_ms[1:]), dist, dev)
    e2e = {"value": world * FRAMES_PER_STEP / (e2e_step / 1000.0), "unit": "frames/s",
           "h2d_bytes_per_step": FRAMES_PER_STEP * 9 * 2 * 8,
           "d2h_bytes_per_step": FRAMES_PER_STEP * N_PIX * N_PIX * 4,
           "path": "Atmosphere.frames_host(dt, 2000): all frames delivered to pinned host "
                   "memory (chunk copies overlapped with rendering), wall clock; per-frame "
                   "shifts travel as kernel parameters"}

    # ---- Monte-Carlo screens/s: Atmosphere.sample(64) at 512^2
    mc_out = None
    for _ in range(3):
        mc_out = atm.sample(MC_BATCH)
    barrier()
    reps = 20
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        mc_out = atm.sample(MC_BATCH)
    e1.record(stream)
    torch.cuda.synchronize()
    mc_sps = world * reps * MC_BATCH / (e0.elapsed_time(e1) / 1000.0)
    # end to end: Atmosphere.sample_host, chunks of 64 drawn while the previous
    # chunk is copied into pinned host memory
    mc_host = torch.empty((5 * MC_BATCH, N_PIX, N_PIX), dtype=torch.float32, pin_memory=True)
    atm.sample_host(2 * MC_BATCH, out=mc_host[:2 * MC_BATCH], chunk=MC_BATCH)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    atm.sample_host(5 * MC_BATCH, out=mc_host, chunk=MC_BATCH)
    torch.cuda.synchronize()
    mc_e2e = world * 5 * MC_BATCH / (time.perf_counter() - t0)

    # ---- roofline of the dominant kernel (live event timing over the timed region)
    hbm, _tf, peak_kind = peaks()
    top = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (1, 1.0))
    name, (nlaunch, kms) = top
    ns, L = N_PIX, 9
    frames_per_launch = FRAMES_PER_STEP * args.steps / max(1, nlaunch)
    pairs = frames_per_launch / 2.0
    blocks = np.ceil(frames_per_launch / 64.0)  # recurrence anchor blocks (64 frames) per launch
    log2n = np.log2(ns)
    # algorithmic bytes and FP32 flops per launch: the rows kernel reads every
    # layer's spectrum once per anchor block and writes the packed intermediate;
    # the column kernel reads it and writes two float32 frames per pair
    algo = {
        "k_frame_rows_uniform": (blocks * L * ns * ns * 8 + pairs * ns * ns * 8,
                                 frames_per_launch * (L * 8 * ns * ns)
                                 + pairs * 5 * ns * ns * log2n),
        "k_frame_rows": (pairs * (L * ns * ns * 8 + ns * ns * 8),
                         frames_per_launch * L * 14 * ns * ns + pairs * 5 * ns * ns * log2n),
        "k_pair_cols": (pairs * (ns * ns * 8 + 2 * N_PIX * N_PIX * 4),
                        pairs * 5 * ns * ns * log2n + frames_per_launch * 4 * LEVELS * ns * ns),
    }.get(name, (0.0, 0.0))
    sec = kms / nlaunch / 1000.0
    achieved = algo[0] / sec / 1e9 if algo[0] else None
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12  # TFLOP/s, SIMT FP32 at max SM clock (nominal)
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": (achieved / hbm) if achieved else None,
                "traffic": captured_traffic(name, frames_per_launch),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                  "64-frame launch (profiles/dram_traffic.json), scaled to "
                                  "the frames per launch; L2-resident writes not counted",
                "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})",
                "kernel_timing": "CUDA events around every launch of these kernels in the "
                                 "chunk-by-chunk pass of the same windows (the graph replays "
                                 "the same kernels)",
                "algorithmic_bytes_per_launch": algo[0],
                "fp32_tflops": algo[1] / sec / 1e12 if algo[1] else None,
                "fp32_frac_of_nominal": (algo[1] / sec / 1e12 / fp32_peak) if algo[1] else None,
                "kernel_share": {k: round(v[1] / max(1e-9, sum(x[1] for x in prof.values())), 4)
                                 for k, v in prof.items()},
                "kernel_ms_per_launch": {k: v[1] / v[0] for k, v in prof.items()}}
    # the per-frame bytes of the reference's formulation (all L stored spectra read
    # and one frame written per frame), over the whole step; the recurrence here
    # does not re-read the spectra per frame, so this exceeds the DRAM traffic
    ref_bpf = L * ns * ns * 8 + N_PIX * N_PIX * 4
    roofline["reference_formulation"] = {
        "bytes_per_frame": ref_bpf, "achieved_gbs": ref_bpf * value / world / 1e9,
        "frac": ref_bpf * value / world / 1e9 / hbm}

    line = {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": bench_config(world),
        "direct_launches": direct,
        "mc_screens_per_s": mc_sps,
        "mc_e2e_screens_per_s": mc_e2e,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clk,
        "wall_s_timed_region": wall,
    }
    line["generate_256_screens_per_s"] = bench_generate(torch, G)
    # config 1 and Monte-Carlo against HBM: the algorithmic bytes are the
    # float32 screens written (the spectra are generated in registers)
    for key, sps, n_px, prof_note in (
            ("generate_256_roofline", line["generate_256_screens_per_s"], 256,
             "64 screens per call"),
            ("mc_roofline", mc_sps, N_PIX, f"Atmosphere.sample({MC_BATCH})")):
        gbs = sps * n_px * n_px * 4 / 1e9
        line[key] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                     "frac": gbs / hbm, "bytes_per_screen": n_px * n_px * 4,
                     "workload": f"{n_px}^2 screens, {prof_note}",
                     "note": "issue-bound kernels (Philox + Box-Muller + register FFT rows; "
                             "barrier-bound 1024-thread column pass): profiles/"
                             "generate_512_mc.md"}
    line["dft_512_tc_vs_fp32"] = bench_tc_dft(torch)
    if not args.no_extrude:
        line["extrude_1024"] = bench_extrude(torch, G)
    if not args.no_diff:
        line["diff_readout_768"] = bench_diff(torch, G)
    line["ragged_mc_4096"] = bench_ragged(torch)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        fps, sps, cores, done, drawn = cpu_reference(200, MC_BATCH, 12.0)
        line["cpu_baseline"] = {
            "value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
            "mc_screens_per_s": sps,
            "sample": f"{done} frames + {drawn} MC screens of the same workload (bounded "
                      "~12 s), float32 NumPy/SciPy port of Atmosphere._integrate, scipy FFT "
                      "workers=all cores"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
