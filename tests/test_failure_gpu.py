"""Failure detection without a GPU fault: a bounded mbarrier wait that nothing
completes must run out, report through the device error word, and leave the
context usable for the next call."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_error(clear=True):
    from pyturb_gb300 import _lib

    v = C.c_int(-1)
    _lib.call("pt_device_error", C.byref(v), 1 if clear else 0)
    return v.value


def test_bounded_wait_runs_out_and_reports():
    import pyturb_gb300 as G
    from pyturb_gb300 import _lib
    from pyturb_gb300.backend import to_numpy

    _device_error(clear=True)
    out = C.c_int(-1)
    _lib.call("pt_selftest_wait_timeout", 1000, C.byref(out))
    assert out.value == 1
    assert _device_error(clear=True) & 1
    # the context still works and no new error is recorded
    g = G.PhaseScreen(n=256, pixel_scale=0.02, r0=0.1, seed=3)
    s = to_numpy(g.generate(4))
    assert np.all(np.isfinite(s))
    assert _device_error(clear=True) == 0


def test_selftest_rejects_bad_limits():
    from pyturb_gb300 import _lib

    out = C.c_int(0)
    with pytest.raises(ValueError):
        _lib.call("pt_selftest_wait_timeout", 0, C.byref(out))
