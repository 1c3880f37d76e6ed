"""The allocation-free inverse FFT entry point, called through the C-ABI.

``pt_ifft2_noalloc`` serves callers that cannot call cudaMalloc (a host
framework that owns all device memory, or a process that must not grow after
start-up): it takes no plan and no workspace, and its scratch is a fixed
file-scope device array. It must give the same transform as the allocating
``pt_ifft2`` — within the tolerance of ``tests/test_fft_gpu.py`` — on two
calls in a row with different sizes (the power-of-two register path, then
the mixed-radix path), so the second call also shows that the shared scratch
left by the first does not leak into it.

This file is named to be collected last: a failure here leaves every other
test already run.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6  # relative L2, as the FFT tests


def _complex_input(rng, batch, n):
    return rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))


def _to_device(x):
    import torch

    return torch.from_numpy(np.stack([x.real, x.imag], -1).astype(np.float32)).cuda()


def _to_host(t):
    o = t.cpu().numpy().astype(np.float64)
    return o[..., 0] + 1j * o[..., 1]


def _with_plan(x):
    import torch

    from pyturb_gb300 import _lib
    from pyturb_gb300.fourier import Grid

    b, n, _ = x.shape
    g = Grid(n, 0.01, np.zeros((0, 3)))
    inp = _to_device(x)
    out = torch.empty_like(inp)
    _lib.call("pt_ifft2", g.handle, inp.data_ptr(), out.data_ptr(), b, g.work.data_ptr(),
              g.work_bytes, torch.cuda.current_stream().cuda_stream)
    return _to_host(out)


def _no_alloc(x):
    import torch

    from pyturb_gb300 import _lib

    b, n, _ = x.shape
    inp = _to_device(x)
    out = torch.empty_like(inp)
    _lib.call("pt_ifft2_noalloc", n, inp.data_ptr(), out.data_ptr(), b,
              torch.cuda.current_stream().cuda_stream)
    return _to_host(out)


def test_no_alloc_ifft2_matches_planned_entry_point_on_two_calls():
    rng = np.random.default_rng(7)
    for n, batch in ((512, 5), (384, 2)):
        x = _complex_input(rng, batch, n)
        ref = _with_plan(x)
        got = _no_alloc(x)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < TOL, (n, err)
        exact = np.fft.ifft2(x) * (n * n)
        assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < TOL


def test_no_alloc_tiny_grids_with_more_images_than_one_launch():
    """ns = 4 and ns = 3 (mixed-radix path) with 70000 images: the scratch
    holds more than 65535 such images, so the call must split them into
    launches that the grid limit allows."""
    rng = np.random.default_rng(8)
    for n in (4, 3):
        x = _complex_input(rng, 70000, n)
        got = _no_alloc(x)
        exact = np.fft.ifft2(x) * (n * n)
        assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < TOL, n


def test_no_alloc_rejects_grids_beyond_its_scratch():
    from pyturb_gb300 import _lib

    with pytest.raises(ValueError, match="1024"):
        _lib.call("pt_ifft2_noalloc", 2048, C.c_void_p(16), C.c_void_p(16), 1, None)
