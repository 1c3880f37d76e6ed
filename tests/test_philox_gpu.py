"""Screens drawn with the kernels' own Philox noise against the float64
oracle fed the same normals (oracle/philox.py), on every transform path of
generate: power-of-two register (64, 256), mixed-radix shared memory (96),
Good-Thomas register (192, 384, 768, 1536 = 3 x 2^k) and the Bluestein form
of the shared-memory passes (202 = 2 x 101, 586 = 2 x 293). Tolerance: relative L2
1e-5 (the device's Box-Muller uses hardware log2 / sqrt / sincos, absolute
error near 1e-6 per normal)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,count", [(64, 5), (256, 4), (96, 7), (192, 3), (384, 4), (768, 3),
                                     (1536, 1), (202, 3), (586, 2)])
def test_device_noise_screens_match_oracle(n, count):
    import oracle
    import pyturb_gb300 as G
    from oracle.philox import PhiloxDraws
    from pyturb_gb300.backend import to_numpy

    from cases import rel_l2

    kw = dict(n=n, pixel_scale=4.0 / n, r0=0.12, L0=20.0, subharmonics=3)
    g = G.PhaseScreen(seed=31, **kw)
    key, call = g._rng.key, g._rng.call
    got = to_numpy(g.generate(count))
    draws = PhiloxDraws(key, call, n, count, 3)
    ref = oracle.OraclePhaseScreen(kw["n"], kw["pixel_scale"], kw["r0"], kw["L0"], 3,
                                   rng=draws).generate(count)
    err = rel_l2(got, ref)
    assert err < 1e-5, err
