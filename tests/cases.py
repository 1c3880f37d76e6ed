"""Shared builders of the golden parity cases.

Each case is defined once by the parameters stored with the golden fixture
(``tests/golden/golden.npz``, made from the reference itself by
``tests/golden/make_golden.py``) and evaluated two ways on the same seeds:
by the float64 oracle (``oracle/``) and by the GPU package with host noise
(``host_noise=numpy.random.default_rng``). The reference draws its normals
from ``numpy.random.default_rng(seed)`` in a fixed order; both evaluations
consume the same streams in that order.
"""

from __future__ import annotations

import json
from functools import lru_cache
from pathlib import Path
from types import SimpleNamespace

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


@lru_cache(maxsize=1)
def golden():
    data = np.load(GOLDEN)
    arrays = {k: data[k] for k in data.files if k != "__meta__"}
    meta = json.loads(str(data["__meta__"]))
    return arrays, meta


def layer_objs(profile):
    return [SimpleNamespace(altitude=a, cn2_fraction=f, wind_speed=v, wind_direction=d, L0=L0)
            for a, f, v, d, L0 in profile]


def _inf(x):
    return np.inf if x is None else x


# ---------------------------------------------------------------- oracle side
def oracle_case(name: str):
    """Evaluate golden case ``name`` with the oracle (float64)."""
    import oracle as O

    arrays, meta = golden()
    rng = np.random.default_rng
    if name.startswith("gen_"):
        m = meta[name]
        g = O.OraclePhaseScreen(m["n"], m["pixel_scale"], m["r0"], _inf(m["L0"]),
                                m["subharmonics"], m.get("power_law", 11 / 3),
                                m.get("inner_scale", 0.0), rng=rng(m["seed"]))
        return g.generate(m["count"])
    if name == "flow_64":
        m = meta[name]
        t = O.OraclePhaseScreen(m["n"], m["pixel_scale"], m["r0"], m["L0"], m["subharmonics"],
                                rng=rng(m["template_seed"]))
        f = O.OracleFlow(t, rng(m["seed"]))
        return np.stack([f.translate(sx, sy) for sx, sy in m["shifts"]])
    if name.startswith("atm"):
        return _oracle_atm(name, meta)
    if name.startswith("ext"):
        return _oracle_ext(name, meta)
    if name.startswith("inf_"):
        m = meta["inf"]
        interp = name.split("_", 1)[1]
        s = O.OracleInfinite(m["n"], m["pixel_scale"], m["r0"], m["L0"], interp=interp,
                             rng=rng(m["seed"]))
        return np.stack([s.screen.copy(), s.step(1).copy(), s.advance(0.37).copy(),
                         s.step(45).copy(), s.advance(2.5).copy()])
    raise KeyError(name)


def _atm_kwargs(m):
    return dict(r0=m["r0"], zenith_angle=m["zenith_angle"], diameter=m["diameter"], n=m["n"],
                subharmonics=m["subharmonics"], seed=m["seed"])


def _oracle_atm(name, meta):
    import oracle as O
    from pyturb_gb300.optics import output_scale

    if name in ("atm_frames", "atm_frames_t", "atm_opd_t0.5", "atm_opd_wl", "atm_sample"):
        m = meta["atm"]
        a = O.OracleAtmosphere(layer_objs(m["profile"]), **_atm_kwargs(m))
        fr = a.frames(0.01, 4)
        if name == "atm_frames":
            return np.stack([f for _, f in fr])
        if name == "atm_frames_t":
            return np.array([t for t, _ in fr])
        if name == "atm_opd_t0.5":
            return a.opd(0.5)
        if name == "atm_opd_wl":
            return a.phase(0.3) * output_scale(500e-9, 1.65e-6)
        a2 = O.OracleAtmosphere(layer_objs(m["profile"]), **_atm_kwargs(m))
        return a2.sample(3)
    if name == "atm_dirs":
        m = meta[name]
        a = O.OracleAtmosphere(layer_objs(m["profile"]), field_of_view=m["field_of_view"],
                               **_atm_kwargs(m))
        return a.opd(m["t"], directions=m["directions"])
    if name in ("atm2_sample", "atm2_opd_wl"):
        m = meta["atm2"]
        a = O.OracleAtmosphere(layer_objs(m["profile"]), **_atm_kwargs(m))
        if name == "atm2_sample":
            return a.sample(2)
        return a.phase(0.1) * output_scale(500e-9, 2.2e-6, "ciddor", 0.3)
    if name.startswith("atm_lgs_"):
        m = meta["atm_lgs"]
        interp = name.rsplit("_", 1)[1]
        a = O.OracleAtmosphere(layer_objs(m["profile"]), lgs_altitude=m["lgs_altitude"],
                               interp=interp, **_atm_kwargs(m))
        return np.stack([f for _, f in a.frames(m["dt"], m["steps"])])
    if name == "atm_boil":
        m = meta[name]
        a = O.OracleAtmosphere(layer_objs(m["profile"]), tau_boil=[_inf(x) for x in m["tau_boil"]],
                               **_atm_kwargs(m))
        return np.stack([f for _, f in a.frames(m["dt"], m["steps"])])
    raise KeyError(name)


def ext_layer_args(m, field_of_view=0.0, lgs_altitude=None):
    """The ExtrudedAtmosphere arguments Atmosphere(engine='extrude') derives
    (``src/pyturb/atmosphere.py:365-530``), including the seed spawning."""
    lys = layer_objs(m["profile"])
    frac = np.array([ly.cn2_fraction for ly in lys], dtype=float)
    frac /= frac.sum()
    cos_z = np.cos(np.deg2rad(m["zenith_angle"]))
    air = 1.0 / cos_z
    r0_los = m["r0"] * cos_z ** (3.0 / 5.0)
    dx = m["diameter"] / m["n"]
    master = np.random.SeedSequence(m["seed"])
    children = master.spawn(len(lys))
    seeds = [int(c.spawn(3)[2].generate_state(1)[0]) for c in children]
    master.spawn(1)  # the spectral engine's boil stream
    ext_boil_seed = int(master.spawn(1)[0].generate_state(1)[0])
    alt = [ly.altitude * air for ly in lys]
    wind = [(ly.wind_speed * np.cos(np.deg2rad(ly.wind_direction)),
             ly.wind_speed * np.sin(np.deg2rad(ly.wind_direction))) for ly in lys]
    arc = np.pi / (180 * 3600)
    return dict(n=m["n"], pixel_scale=dx, layer_r0=[r0_los * f ** (-0.6) for f in frac],
                layer_L0=[ly.L0 for ly in lys], layer_wind=wind, layer_altitude_los=alt,
                field_of_view_pix=[a * np.tan(field_of_view * arc) / dx for a in alt],
                lgs_altitude_los=None if lgs_altitude is None else lgs_altitude * air,
                seeds=seeds, boil_seed=ext_boil_seed)


def _oracle_ext(name, meta):
    import oracle as O

    arc = np.pi / (180 * 3600)
    if name == "ext_dirs_lgs":
        m = meta[name]
        e = O.OracleExtruded(**ext_layer_args(m, m["field_of_view"], m["lgs_altitude"]))
        e.set_time(m["t"])
        return np.stack([e.integrate(np.tan(a * arc), np.tan(b * arc))
                         for a, b in m["directions"]]) * (500e-9 / (2 * np.pi))
    if name == "ext_boil":
        m = meta[name]
        e = O.OracleExtruded(interp="linear", tau_boil=m["tau_boil"], **ext_layer_args(m))
        out, t = [], 0.0
        for _ in range(m["steps"]):  # Atmosphere.frames: frame, then the boil step
            e.set_time(t)
            out.append(e.integrate() * (500e-9 / (2 * np.pi)))
            e.boil_step(m["dt"])
            t += m["dt"]
        return np.stack(out)
    m = meta["ext"]
    interp = name.split("_", 1)[1]
    e = O.OracleExtruded(interp=interp, **ext_layer_args(m))
    out, t = [], 0.0
    for _ in range(m["steps"]):
        e.set_time(t)
        out.append(e.integrate() * (500e-9 / (2 * np.pi)))
        t += m["dt"]
    return np.stack(out)


# ---------------------------------------------------------------- GPU side
def gpu_case(name: str):
    """Evaluate golden case ``name`` with pyturb_gb300 on the GPU (host noise)."""
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    arrays, meta = golden()
    rng = np.random.default_rng
    if name.startswith("gen_"):
        m = meta[name]
        g = G.PhaseScreen(m["n"], m["pixel_scale"], m["r0"], _inf(m["L0"]),
                          subharmonics=m["subharmonics"],
                          power_law=m.get("power_law", 11 / 3),
                          inner_scale=m.get("inner_scale", 0.0), seed=m["seed"],
                          host_noise=rng)
        return to_numpy(g.generate(m["count"])).astype(np.float64)
    if name == "flow_64":
        m = meta[name]
        t = G.PhaseScreen(m["n"], m["pixel_scale"], m["r0"], m["L0"],
                          subharmonics=m["subharmonics"], seed=m["template_seed"],
                          host_noise=rng)
        f = G.FourierFlowScreen(t, seed=m["seed"])
        return np.stack([to_numpy(f.translate(sx, sy)) for sx, sy in m["shifts"]]).astype(float)
    if name.startswith("atm"):
        return _gpu_atm(name, meta)
    if name.startswith("ext"):
        return _gpu_ext(name, meta)
    if name.startswith("inf_"):
        m = meta["inf"]
        interp = name.split("_", 1)[1]
        s = G.InfinitePhaseScreen(m["n"], m["pixel_scale"], m["r0"], m["L0"], interp=interp,
                                  seed=m["seed"], host_noise=rng)
        seq = [to_numpy(s.screen), to_numpy(s.step()), to_numpy(s.advance(0.37)),
               to_numpy(s.step(45)), to_numpy(s.advance(2.5))]
        return np.stack(seq).astype(float)
    raise KeyError(name)


def _gpu_layers(profile):
    import pyturb_gb300 as G

    return [G.Layer(a, f, v, d, L0) for a, f, v, d, L0 in profile]


def _gpu_atm(name, meta):
    import warnings

    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    rng = np.random.default_rng
    np_ = lambda x: to_numpy(x).astype(np.float64)  # noqa: E731
    if name in ("atm_frames", "atm_frames_t", "atm_opd_t0.5", "atm_opd_wl", "atm_sample"):
        m = meta["atm"]
        a = G.Atmosphere(_gpu_layers(m["profile"]), host_noise=rng, **_atm_kwargs(m))
        fr = [(t, np_(f)) for t, f in a.frames(dt=0.01, steps=4)]
        if name == "atm_frames":
            return np.stack([f for _, f in fr])
        if name == "atm_frames_t":
            return np.array([t for t, _ in fr])
        if name == "atm_opd_t0.5":
            return np_(a.opd(0.5))
        if name == "atm_opd_wl":
            return np_(a.opd(0.3, wavelength=1.65e-6))
        return np_(a.sample(3))
    if name == "atm_dirs":
        m = meta[name]
        a = G.Atmosphere(_gpu_layers(m["profile"]), field_of_view=m["field_of_view"],
                         host_noise=rng, **_atm_kwargs(m))
        return np_(a.opd(m["t"], directions=m["directions"]))
    if name in ("atm2_sample", "atm2_opd_wl"):
        m = meta["atm2"]
        a = G.Atmosphere(_gpu_layers(m["profile"]), dispersion="ciddor", wet_fraction=0.3,
                         host_noise=rng, **_atm_kwargs(m))
        if name == "atm2_sample":
            return np_(a.sample(2))
        return np_(a.opd(0.1, wavelength=2.2e-6))
    if name.startswith("atm_lgs_"):
        m = meta["atm_lgs"]
        interp = name.rsplit("_", 1)[1]
        a = G.Atmosphere(_gpu_layers(m["profile"]), lgs_altitude=m["lgs_altitude"],
                         interp=interp, host_noise=rng, **_atm_kwargs(m))
        return np.stack([np_(f) for _, f in a.frames(dt=m["dt"], steps=m["steps"])])
    if name == "atm_boil":
        m = meta[name]
        a = G.Atmosphere(_gpu_layers(m["profile"]), tau_boil=[_inf(x) for x in m["tau_boil"]],
                         host_noise=rng, **_atm_kwargs(m))
        return np.stack([np_(f) for _, f in a.frames(dt=m["dt"], steps=m["steps"])])
    raise KeyError(name)


def _gpu_ext(name, meta):
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    rng = np.random.default_rng
    np_ = lambda x: to_numpy(x).astype(np.float64)  # noqa: E731
    kw = lambda m: dict(r0=m["r0"], zenith_angle=m["zenith_angle"],  # noqa: E731
                        diameter=m["diameter"], n=m["n"], seed=m["seed"])
    if name == "ext_dirs_lgs":
        m = meta[name]
        a = G.Atmosphere(_gpu_layers(m["profile"]), engine="extrude",
                         field_of_view=m["field_of_view"], lgs_altitude=m["lgs_altitude"],
                         host_noise=rng, **kw(m))
        return np_(a.opd(m["t"], directions=m["directions"]))
    if name == "ext_boil":
        m = meta[name]
        a = G.Atmosphere(_gpu_layers(m["profile"]), engine="extrude", interp="linear",
                         tau_boil=m["tau_boil"], host_noise=rng, **kw(m))
        return np.stack([np_(f) for _, f in a.frames(dt=m["dt"], steps=m["steps"])])
    m = meta["ext"]
    interp = name.split("_", 1)[1]
    a = G.Atmosphere(_gpu_layers(m["profile"]), engine="extrude", interp=interp,
                     host_noise=rng, **kw(m))
    return np.stack([np_(f) for _, f in a.frames(dt=m["dt"], steps=m["steps"])])


CASES = ["gen_64", "gen_48", "gen_37", "gen_64_nosh", "gen_32_kolmo", "gen_60_vk", "flow_64",
         "atm_frames", "atm_frames_t", "atm_opd_t0.5", "atm_opd_wl", "atm_sample", "atm_dirs",
         "atm2_sample", "atm2_opd_wl", "atm_lgs_cubic", "atm_lgs_linear", "atm_lgs_lanczos",
         "atm_boil", "ext_cubic", "ext_linear", "ext_lanczos", "ext_dirs_lgs", "ext_boil", "inf_cubic",
         "inf_linear", "inf_lanczos"]


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
