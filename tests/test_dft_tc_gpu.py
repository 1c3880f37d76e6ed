"""The tensor-core 512-point DFT form (pt_ifft2_tc) against float64 numpy
and against the FP32 register FFT (pt_ifft2), through the C-ABI: relative L2
within 1e-5 of float64, in place and out of place."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _dev(x):
    import torch

    return torch.from_numpy(np.stack([x.real, x.imag], -1).astype(np.float32)).cuda()


def _host(t):
    o = t.cpu().numpy().astype(np.float64)
    return o[..., 0] + 1j * o[..., 1]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tc_dft_matches_float64_and_the_fp32_fft():
    import torch

    from pyturb_gb300 import _lib
    from pyturb_gb300.fourier import Grid

    rng = np.random.default_rng(11)
    n, batch = 512, 3
    # a coloured spectrum like the screens' (steep power law) and white noise
    f = np.fft.fftfreq(n)
    amp = (f[:, None] ** 2 + f[None, :] ** 2 + 1e-4) ** (-11.0 / 12.0)
    for scale in (amp, np.ones((n, n))):
        x = (rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))) * scale
        exact = np.fft.ifft2(x) * (n * n)
        inp = _dev(x)
        out = torch.empty_like(inp)
        s = torch.cuda.current_stream().cuda_stream
        _lib.call("pt_ifft2_tc", n, inp.data_ptr(), out.data_ptr(), batch, s)
        e_tc = _rel(_host(out), exact)
        _lib.call("pt_ifft2_tc", n, inp.data_ptr(), inp.data_ptr(), batch, s)  # in place
        assert _rel(_host(inp), _host(out)) == 0.0
        g = Grid(n, 0.01, np.zeros((0, 3)))
        ref = torch.empty_like(out)
        _lib.call("pt_ifft2", g.handle, _dev(x).data_ptr(), ref.data_ptr(), batch,
                  g.work.data_ptr(), g.work_bytes, s)
        e_fft = _rel(_host(ref), exact)
        print(f"relative L2 vs float64: tensor-core DFT {e_tc:.2e}, FP32 FFT {e_fft:.2e}")
        assert e_tc < TOL
    # every bounded barrier wait of the products completed
    import ctypes as C

    err = C.c_int(-1)
    _lib.call("pt_device_error", C.byref(err), 1)
    assert err.value == 0


def test_tc_dft_refuses_other_sizes():
    from pyturb_gb300 import _lib

    with pytest.raises(RuntimeError, match="512"):
        _lib.call("pt_ifft2_tc", 256, 16, 16, 1, None)
