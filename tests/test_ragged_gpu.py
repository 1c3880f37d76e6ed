"""Ragged Monte-Carlo ensembles: each screen is r0^(-5/6) times the unit-r0
screen of its (n, dx, L0) group, drawn with the group's Philox key."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_screens_equal_scaled_unit_screens():
    import torch

    from pyturb_gb300 import _lib
    from pyturb_gb300.backend import dptr, stream_handle
    from pyturb_gb300.ragged import RaggedEnsemble

    sizes = [64, 128, 64, 96, 128, 64, 96]
    r0 = [0.08, 0.1, 0.12, 0.15, 0.2, 0.25, 0.1]
    L0 = [10.0, 25.0, 10.0, 50.0, 25.0, 25.0, 50.0]
    ens = RaggedEnsemble(sizes, r0, L0, pixel_scale=1.0 / 64, subharmonics=3, seed=11)
    assert ens.n_groups == 4
    buf = ens.generate().clone()
    call = ens._rng.call - 1  # the counter the draw used
    for g, key in zip(ens.groups, ens._keys):
        unit = torch.empty((len(g.members), g.n, g.n), device="cuda")
        _lib.call("pt_generate", g.grid.handle, len(g.members), dptr(g.amplitude),
                  dptr(g.sh_amp), None, None, key, call, 0, g.n, 1.0, 0, dptr(unit),
                  dptr(ens.work), ens.work_bytes, stream_handle())
        for k, i in enumerate(g.members):
            got = ens.screen(i).double().cpu().numpy()
            o = int(ens.offsets[i])
            assert np.array_equal(got, buf[o:o + g.n * g.n].view(g.n, g.n).double().cpu().numpy())
            want = unit[k].double().cpu().numpy() * r0[i] ** (-5.0 / 6.0)
            err = np.linalg.norm(got - want) / np.linalg.norm(want)
            assert err < 1e-6, (i, err)


def test_new_draws_differ_and_stay_finite():
    from pyturb_gb300.ragged import RaggedEnsemble

    ens = RaggedEnsemble([32, 48, 32], 0.1, 25.0, seed=3)
    a = ens.generate().clone()
    b = ens.generate().clone()
    assert bool(a.isfinite().all()) and bool(b.isfinite().all())
    assert float((a - b).abs().max()) > 0.0


def test_argument_errors():
    from pyturb_gb300.ragged import RaggedEnsemble

    with pytest.raises(ValueError):
        RaggedEnsemble([], 0.1, 25.0)
    with pytest.raises(ValueError):
        RaggedEnsemble([64], -0.1, 25.0)
    with pytest.raises(ValueError):
        RaggedEnsemble([64], 0.1, float("inf"))
