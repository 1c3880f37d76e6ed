"""Autotuned schedules: every candidate radix plan and column variant gives the
same screens, and cached choices are reused."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [384, 96, 75])
def test_every_radix_plan_gives_the_same_screens(n):
    import torch

    from pyturb_gb300 import PhaseScreen, tuning

    ps = PhaseScreen(n=n, pixel_scale=0.02, r0=0.1, L0=20.0, subharmonics=2, seed=4)
    out = torch.empty((6, n, n), device="cuda")
    plans = tuning.radix_plans(n)
    default = tuning.grid_radices(ps._grid)
    ref = None
    for plan in [default] + plans:
        tuning.set_grid_radices(ps._grid, plan)
        ps._rng.call = 0
        ps._generate_into(out, 6, 0, n, 1.0, False)
        got = out.double().cpu().numpy()
        if ref is None:
            ref = got
        else:
            err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
            assert err < 2e-6, (plan, err)


def test_cols_variants_agree():
    import torch

    from pyturb_gb300 import PhaseScreen, _lib

    ps = PhaseScreen(n=256, pixel_scale=0.02, r0=0.1, L0=20.0, subharmonics=3, seed=4)
    out = torch.empty((8, 256, 256), device="cuda")
    res = []
    for v in (0, 1):
        _lib.call("pt_grid_set_cols_variant", ps._grid.handle, v)
        ps._rng.call = 0
        ps._generate_into(out, 8, 0, 256, 1.0, False)
        res.append(out.double().cpu().numpy())
    assert np.linalg.norm(res[0] - res[1]) / np.linalg.norm(res[0]) < 1e-6


def test_autotune_is_cached_and_keeps_the_stream(tmp_path, monkeypatch):
    from pyturb_gb300 import PhaseScreen, tuning

    monkeypatch.setenv("PYTURB_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    ps = PhaseScreen(n=96, pixel_scale=0.02, r0=0.1, L0=20.0, subharmonics=2, seed=4)
    call = ps._rng.call
    choice = ps.autotune(4)
    assert ps._rng.call == call and "radices" in choice
    assert tuple(choice["radices"]) == tuning.grid_radices(ps._grid)
    assert any("radices|n=96|batch=4" in k for k in tuning._load())
    ps2 = PhaseScreen(n=96, pixel_scale=0.02, r0=0.1, L0=20.0, subharmonics=2, seed=4)
    assert ps2.autotune(4) == choice          # from the cache
    # generate at 3 x 2^k (here 384) has no radix plan to tune
    assert PhaseScreen(n=384, pixel_scale=0.02, r0=0.1, L0=20.0, seed=4).autotune(4) == {}
    with pytest.raises(ValueError):
        PhaseScreen(n=64, pixel_scale=0.02, r0=0.1, host_noise=np.random.default_rng).autotune(2)


def test_frame_loop_auto_branches(tmp_path, monkeypatch):
    import warnings

    import pyturb_gb300 as G

    warnings.simplefilter("ignore")
    monkeypatch.setenv("PYTURB_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    layers = [G.Layer(0.0, 0.6, 9.0, 20.0, 25.0), G.Layer(5000.0, 0.4, 15.0, 100.0, 25.0)]
    atm = G.Atmosphere(layers, r0=0.15, diameter=2.0, n=64, seed=3, frames_chunk=16)
    loop = atm.frame_loop(1e-3, 40, branches="auto")
    assert 1 <= loop.branches <= 4
    got = loop.render(0.2).double().cpu().numpy()
    want = atm.render(0.2 + loop.times).double().cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 2e-6


def test_ragged_autotune_matches_untuned(tmp_path, monkeypatch):
    from pyturb_gb300.ragged import RaggedEnsemble

    monkeypatch.setenv("PYTURB_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    sizes, r0, L0 = [96, 64, 96, 256], [0.1, 0.12, 0.2, 0.15], [10.0, 25.0, 10.0, 50.0]
    a = RaggedEnsemble(sizes, r0, L0, seed=9).generate().double().cpu().numpy()
    tuned = RaggedEnsemble(sizes, r0, L0, seed=9, autotune=True)
    b = tuned.generate().double().cpu().numpy()
    assert tuned.tuning
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 2e-6
