"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs jacotay7/pyturb (imported from its source tree, default
/root/reference/src, override with PYTURB_REF_SRC) in float64 on fixed seeds
and stores each case's parameters and outputs in ``golden.npz``. Only
outputs are stored: both the oracle and the GPU path regenerate the random
normals from the same seeds with ``numpy.random.default_rng``, in the
reference's draw order.

Run in the build container (the reference is not present on GPU machines):
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import os
import sys
import warnings
from pathlib import Path

import numpy as np

REF = os.environ.get("PYTURB_REF_SRC", "/root/reference/src")
OUT = Path(__file__).resolve().parent / "golden.npz"

# one small atmosphere profile shared by the cases: (altitude, cn2, speed, direction, L0)
PROFILE = [(0.0, 0.6, 9.0, 20.0, 25.0), (4000.0, 0.25, 17.0, 135.0, 25.0),
           (11000.0, 0.15, 28.0, 250.0, 25.0)]
PROFILE_2L0 = [(0.0, 0.6, 9.0, 20.0, 25.0), (4000.0, 0.25, 17.0, 135.0, 10.0),
               (11000.0, 0.15, 28.0, 250.0, 25.0)]


def main() -> None:
    sys.path.insert(0, REF)
    import pyturb
    from pyturb.extrude import ExtrudedAtmosphere
    from pyturb.flow import FourierFlowScreen

    warnings.simplefilter("ignore")
    cases = {}
    meta = {}

    def layers(prof):
        return [pyturb.Layer(a, f, v, d, L0) for a, f, v, d, L0 in prof]

    # --- PhaseScreen.generate: even/odd counts, mixed radix, prime size, no subharmonics, Kolmogorov
    gen_cases = [
        ("gen_64", dict(n=64, pixel_scale=0.05, r0=0.1, L0=25.0, subharmonics=3, seed=11), 5),
        ("gen_48", dict(n=48, pixel_scale=0.04, r0=0.12, L0=20.0, subharmonics=2, seed=5), 4),
        ("gen_37", dict(n=37, pixel_scale=0.06, r0=0.15, L0=25.0, subharmonics=1, seed=2), 3),
        ("gen_64_nosh", dict(n=64, pixel_scale=0.05, r0=0.1, L0=25.0, subharmonics=0, seed=3), 2),
        ("gen_32_kolmo", dict(n=32, pixel_scale=0.05, r0=0.1, L0=np.inf, subharmonics=3,
                              seed=9), 1),
        ("gen_60_vk", dict(n=60, pixel_scale=0.05, r0=0.1, L0=25.0, subharmonics=8, seed=13,
                           power_law=3.4, inner_scale=0.02), 2),
    ]
    for name, kw, count in gen_cases:
        g = pyturb.PhaseScreen(dtype="float64", **kw)
        cases[name] = np.asarray(g.generate(count))
        meta[name] = dict(kind="generate", count=count, **{k: (None if v == np.inf else v)
                                                           for k, v in kw.items()})

    # --- FourierFlowScreen.translate
    tmpl = pyturb.PhaseScreen(n=64, pixel_scale=0.05, r0=0.1, L0=25.0, subharmonics=3, seed=1,
                              dtype="float64")
    flow = FourierFlowScreen(tmpl, seed=4)
    shifts = [(0.37, -1.2), (100.0, 55.5), (0.0, 0.0)]
    cases["flow_64"] = np.stack([flow.translate(sx, sy) for sx, sy in shifts])
    meta["flow_64"] = dict(kind="flow", n=64, pixel_scale=0.05, r0=0.1, L0=25.0,
                           subharmonics=3, template_seed=1, seed=4, shifts=shifts)

    # --- Atmosphere, spectral engine
    atm_kw = dict(r0=0.12, zenith_angle=30.0, diameter=2.0, n=64, subharmonics=3, seed=7)
    atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", **atm_kw)
    fr = list(atm.frames(dt=0.01, steps=4))
    cases["atm_frames"] = np.stack([f for _, f in fr])
    cases["atm_frames_t"] = np.array([t for t, _ in fr])
    cases["atm_opd_t0.5"] = np.asarray(atm.opd(0.5))
    cases["atm_opd_wl"] = np.asarray(atm.opd(0.3, wavelength=1.65e-6))
    cases["atm_sample"] = np.asarray(atm.sample(3))
    meta["atm"] = dict(kind="atmosphere", profile=PROFILE, **atm_kw)

    atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", field_of_view=20.0, **atm_kw)
    dirs = [(0.0, 0.0), (10.0, -5.0), (-12.0, 3.0)]
    cases["atm_dirs"] = np.asarray(atm.opd(0.2, directions=dirs))
    meta["atm_dirs"] = dict(kind="atmosphere", profile=PROFILE, field_of_view=20.0,
                            directions=dirs, t=0.2, **atm_kw)

    atm = pyturb.Atmosphere(layers(PROFILE_2L0), dtype="float64", dispersion="ciddor",
                            wet_fraction=0.3, **atm_kw)
    cases["atm2_sample"] = np.asarray(atm.sample(2))
    cases["atm2_opd_wl"] = np.asarray(atm.opd(0.1, wavelength=2.2e-6))
    meta["atm2"] = dict(kind="atmosphere", profile=PROFILE_2L0, dispersion="ciddor",
                        wet_fraction=0.3, **atm_kw)

    for interp in ("cubic", "linear", "lanczos"):
        atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", lgs_altitude=90e3,
                                interp=interp, **atm_kw)
        cases[f"atm_lgs_{interp}"] = np.stack([f for _, f in atm.frames(dt=0.02, steps=2)])
    meta["atm_lgs"] = dict(kind="atmosphere", profile=PROFILE, lgs_altitude=90e3, dt=0.02,
                           steps=2, **atm_kw)

    atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", tau_boil=[0.05, 0.1, np.inf],
                            **atm_kw)
    cases["atm_boil"] = np.stack([f for _, f in atm.frames(dt=0.01, steps=3)])
    meta["atm_boil"] = dict(kind="atmosphere", profile=PROFILE, tau_boil=[0.05, 0.1, None],
                            dt=0.01, steps=3, **atm_kw)

    # --- Atmosphere, extrusion engine (runs long enough to compact the rings)
    ext_kw = dict(r0=0.12, zenith_angle=0.0, diameter=1.0, n=32, seed=21)
    for interp in ("cubic", "linear", "lanczos"):
        atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", engine="extrude",
                                interp=interp, **ext_kw)
        cases[f"ext_{interp}"] = np.stack([f for _, f in atm.frames(dt=0.04, steps=8)])
    meta["ext"] = dict(kind="extrude", profile=PROFILE, dt=0.04, steps=8, **ext_kw)
    # boiling on the extrusion engine: two boiling layers and one frozen
    tau = [0.08, float("inf"), 0.2]
    atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", engine="extrude", interp="linear",
                            tau_boil=tau, **ext_kw)
    cases["ext_boil"] = np.stack([f for _, f in atm.frames(dt=0.04, steps=6)])
    meta["ext_boil"] = dict(kind="extrude", profile=PROFILE, dt=0.04, steps=6, tau_boil=tau,
                            **ext_kw)
    atm = pyturb.Atmosphere(layers(PROFILE), dtype="float64", engine="extrude",
                            field_of_view=30.0, lgs_altitude=90e3, **ext_kw)
    cases["ext_dirs_lgs"] = np.asarray(atm.opd(0.05, directions=[(0.0, 0.0), (20.0, -10.0)]))
    meta["ext_dirs_lgs"] = dict(kind="extrude", profile=PROFILE, field_of_view=30.0,
                                lgs_altitude=90e3, t=0.05,
                                directions=[(0.0, 0.0), (20.0, -10.0)], **ext_kw)

    # --- InfinitePhaseScreen
    for interp in ("cubic", "linear", "lanczos"):
        inf = pyturb.InfinitePhaseScreen(n=32, pixel_scale=0.05, r0=0.1, L0=20.0, seed=3,
                                         interp=interp, dtype="float64")
        seq = [np.asarray(inf.screen), np.asarray(inf.step()), np.asarray(inf.advance(0.37)),
               np.asarray(inf.step(45)), np.asarray(inf.advance(2.5))]
        cases[f"inf_{interp}"] = np.stack(seq)
    meta["inf"] = dict(kind="infinite", n=32, pixel_scale=0.05, r0=0.1, L0=20.0, seed=3,
                       ops=["screen", "step", "advance 0.37", "step 45", "advance 2.5"])

    cases["__meta__"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **cases)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(cases) - 1} arrays)")


if __name__ == "__main__":
    main()
