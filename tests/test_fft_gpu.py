"""The shared-memory Stockham inverse FFT against numpy (mixed radix, primes,
the Bluestein form for large prime factors, batches larger than one internal
chunk)."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ifft2_gpu(x):
    import torch

    from pyturb_gb300 import _lib
    from pyturb_gb300.fourier import Grid

    b, n, _ = x.shape
    g = Grid(n, 0.01, np.zeros((0, 3)))
    inp = torch.from_numpy(np.stack([x.real, x.imag], -1).astype(np.float32)).cuda()
    out = torch.empty_like(inp)
    _lib.call("pt_ifft2", g.handle, inp.data_ptr(), out.data_ptr(), b, g.work.data_ptr(),
              g.work_bytes, torch.cuda.current_stream().cuda_stream)
    o = out.cpu().numpy().astype(np.float64)
    return o[..., 0] + 1j * o[..., 1]


# 127, 202 = 2 x 101, 586 = 2 x 293, 1031 and 1447 (prime factors above 61)
# take the Bluestein form; 37 and 121 = 11^2 the direct-sum stages
@pytest.mark.parametrize("n", [2, 3, 8, 12, 30, 37, 49, 64, 96, 121, 127, 128, 202, 256, 384,
                               512, 586, 768, 1024, 1031, 1447, 2048])
def test_ifft2_matches_numpy(n):
    rng = np.random.default_rng(n)
    batch = 3 if n <= 1024 else 1
    x = rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))
    ref = np.fft.ifft2(x) * (n * n)
    got = _ifft2_gpu(x)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 2e-6, err


def test_ifft2_batch_beyond_chunk():
    n = 512
    rng = np.random.default_rng(0)
    x = rng.standard_normal((70, n, n)) + 1j * rng.standard_normal((70, n, n))
    got = _ifft2_gpu(x)
    ref = np.fft.ifft2(x) * (n * n)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-6
