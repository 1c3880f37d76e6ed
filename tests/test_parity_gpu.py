"""GPU parity: the GB300 path against the reference's own float64 outputs
(golden fixtures) and against the float64 oracle at the benchmark sizes,
on the same seeds and the same host normals. Tolerance: relative L2 error
1e-5 (float32 GPU result vs float64 reference)."""

import warnings

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.mark.parametrize("name", cases.CASES)
def test_gpu_matches_reference_fixture(name):
    arrays, _ = cases.golden()
    got = cases.gpu_case(name)
    ref = arrays[name]
    assert got.shape == ref.shape
    assert cases.rel_l2(got, ref) < TOL, cases.rel_l2(got, ref)


def test_generate_config1_shape_vs_oracle():
    """PhaseScreen.generate(64), n=256, D=8 m, r0=0.15, L0=25, 3 subharmonic levels."""
    import oracle
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    kw = dict(n=256, pixel_scale=8.0 / 256, r0=0.15, L0=25.0, subharmonics=3)
    g = G.PhaseScreen(seed=123, host_noise=np.random.default_rng, **kw)
    got = to_numpy(g.generate(64))
    ref = oracle.OraclePhaseScreen(kw["n"], kw["pixel_scale"], kw["r0"], kw["L0"], 3,
                                   rng=np.random.default_rng(123)).generate(64)
    assert got.shape == (64, 256, 256) and got.dtype == np.float32
    assert cases.rel_l2(got, ref) < TOL
    # second call continues the stream in the reference's order
    got2 = to_numpy(g.generate(3))
    o = oracle.OraclePhaseScreen(kw["n"], kw["pixel_scale"], kw["r0"], kw["L0"], 3,
                                 rng=np.random.default_rng(123))
    o.generate(64)
    assert cases.rel_l2(got2, o.generate(3)) < TOL


@pytest.mark.parametrize("n,count", [(1024, 19), (64, 601)])
def test_generate_chunk_boundaries_vs_oracle(n, count):
    """Batches spanning several internal chunks (8 transforms per chunk at
    1024^2, 256 at 64^2), odd counts so the last transform carries one screen."""
    import oracle
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    kw = dict(n=n, pixel_scale=4.0 / n, r0=0.1, L0=20.0, subharmonics=2)
    g = G.PhaseScreen(seed=9, host_noise=np.random.default_rng, **kw)
    got = to_numpy(g.generate(count))
    ref = oracle.OraclePhaseScreen(kw["n"], kw["pixel_scale"], kw["r0"], kw["L0"], 2,
                                   rng=np.random.default_rng(9)).generate(count)
    assert got.shape == (count, n, n)
    assert cases.rel_l2(got, ref) < TOL
    per = [cases.rel_l2(got[i], ref[i]) for i in (0, count // 2, count - 1)]
    assert max(per) < 3 * TOL, per


def _config2_layers(seed=0):
    rng = np.random.default_rng(seed)
    h = [0, 500, 1000, 2000, 4000, 8000, 12000, 16000, 20000]
    f = [0.52, 0.10, 0.07, 0.06, 0.05, 0.06, 0.06, 0.05, 0.03]
    v = rng.uniform(5, 30, 9)
    d = rng.uniform(0, 360, 9)
    return [cases.layer_objs([(a, b, c, e, 25.0)])[0] for a, b, c, e in zip(h, f, v, d)]


def test_frames_config2_vs_oracle_long_run():
    """9 layers, n=512, z=30 deg, 3 levels: frames at t = 0, 1 s and 2 s (the
    phase argument range-reduction keeps the error flat in t)."""
    import oracle
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    lys = _config2_layers()
    kw = dict(r0=0.157, zenith_angle=30.0, diameter=8.0, n=512, subharmonics=3, seed=5)
    a = G.Atmosphere([G.Layer(l.altitude, l.cn2_fraction, l.wind_speed, l.wind_direction,
                              l.L0) for l in lys], host_noise=np.random.default_rng, **kw)
    o = oracle.OracleAtmosphere(lys, **kw)
    times = [0.0, 1.0, 2.0]
    got = to_numpy(a.render(times))
    for k, t in enumerate(times):
        err = cases.rel_l2(got[k], o.opd(t))
        assert err < TOL, (t, err)


def test_uniform_chunk_recurrence_vs_oracle():
    """Equally spaced frames take the register-recurrence kernel: check the
    first, anchor-boundary and last frames of full and ragged 64-frame chunks
    against the float64 oracle."""
    import oracle
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    lys = _config2_layers(3)
    kw = dict(r0=0.157, zenith_angle=30.0, diameter=8.0, n=512, subharmonics=3, seed=9)
    a = G.Atmosphere([G.Layer(l.altitude, l.cn2_fraction, l.wind_speed, l.wind_direction,
                              l.L0) for l in lys], host_noise=np.random.default_rng, **kw)
    o = oracle.OracleAtmosphere(lys, **kw)
    times = 1.5 + 1e-3 * np.arange(64 + 37)  # one full chunk and one ragged (odd) chunk
    got = to_numpy(a.render(times))
    for k in (0, 1, 31, 32, 33, 63, 64, 95, 96, 100):
        err = cases.rel_l2(got[k], o.opd(times[k]))
        assert err < TOL, (k, err)


def test_frames_generator_equals_render_and_opd():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    lys = [G.Layer(0, 0.7, 10, 30), G.Layer(5000, 0.3, 25, 200)]
    a = G.Atmosphere(lys, r0=0.15, n=128, diameter=4.0, subharmonics=3, seed=1,
                     frames_chunk=16)
    fr = [(t, to_numpy(f)) for t, f in a.frames(dt=1e-3, steps=37)]
    ts = np.array([t for t, _ in fr])
    assert ts[0] == 0.0 and len(fr) == 37
    ren = to_numpy(a.render(ts))
    for k in (0, 15, 16, 36):
        np.testing.assert_allclose(fr[k][1], ren[k], rtol=0, atol=1e-6 * np.abs(ren).max())
        np.testing.assert_allclose(to_numpy(a.opd(ts[k])), ren[k], rtol=0,
                                   atol=1e-6 * np.abs(ren).max())
    assert a.time == pytest.approx(37e-3)


def test_frames_host_equals_frames_generator():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    lys = [G.Layer(0, 0.7, 10, 30), G.Layer(5000, 0.3, 25, 200)]
    kw = dict(r0=0.15, n=128, diameter=4.0, subharmonics=3, seed=2, frames_chunk=16)
    a = G.Atmosphere(lys, **kw)
    b = G.Atmosphere(lys, **kw)
    host = a.frames_host(dt=1e-3, steps=53)
    ref = np.stack([to_numpy(f) for _, f in b.frames(dt=1e-3, steps=53)])
    assert host.device.type == "cpu" and host.shape == (53, 128, 128)
    np.testing.assert_array_equal(host.numpy(), ref)
    assert a.time == pytest.approx(b.time)


def test_sample_config2_vs_oracle():
    import oracle
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    lys = _config2_layers()
    kw = dict(r0=0.157, zenith_angle=30.0, diameter=8.0, n=512, subharmonics=3, seed=8)
    a = G.Atmosphere([G.Layer(l.altitude, l.cn2_fraction, l.wind_speed, l.wind_direction,
                              l.L0) for l in lys], host_noise=np.random.default_rng, **kw)
    o = oracle.OracleAtmosphere(lys, **kw)
    assert cases.rel_l2(to_numpy(a.sample(6)), o.sample(6)) < TOL


def test_sample_host_equals_repeated_sample():
    """sample_host(count, chunk) delivers the screens of repeated sample(chunk)
    calls into pinned host memory (two L0 groups, a short last chunk)."""
    import torch

    import pyturb_gb300 as G

    lys = _config2_layers(3)
    lys[-1] = cases.layer_objs([(20000, 0.03, 12.0, 40.0, 50.0)])[0]  # a second L0 group
    kw = dict(r0=0.15, zenith_angle=10.0, diameter=4.0, n=128, subharmonics=2, seed=21)
    mk = lambda: G.Atmosphere([G.Layer(l.altitude, l.cn2_fraction, l.wind_speed,
                                       l.wind_direction, l.L0) for l in lys], **kw)
    got = mk().sample_host(22, chunk=8)
    assert got.device.type == "cpu" and got.is_pinned() and tuple(got.shape) == (22, 128, 128)
    a = mk()
    want = torch.cat([a.sample(8).cpu(), a.sample(8).cpu(), a.sample(6).cpu()])
    assert torch.equal(got, want)
