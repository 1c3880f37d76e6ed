"""Validation diagnostics on the device (drop-in for the reductions of
``pyturb.utils`` / ``pyturb.analysis``): the phase structure function, the
least-squares Zernike decomposition and the temporal power spectrum.

The reference brings device arrays to the host and reduces in NumPy
(``src/pyturb/utils.py:159-201``, ``src/pyturb/analysis.py:129-208``). Here
the reductions run where the screens already are; the returned arrays are
NumPy (float64), as the reference's. The Zernike basis is host FP64 setup
(Noll 1976 indexing and normalisation, ``analysis.py:56-128``) and its
pseudo-inverse is cached per (n_modes, n_pixels, diameter).
"""

from __future__ import annotations

from functools import lru_cache
from math import factorial
from typing import Optional, Tuple

import numpy as np

from . import _lib
from .backend import cuda_device, dptr, stream_handle, to_numpy, torch_module

__all__ = ["noll_to_zernike", "zernike_basis", "zernike_decompose", "structure_function",
           "temporal_psd"]


def _device_f32(a):
    """A contiguous float32 CUDA tensor view or copy of ``a``."""
    torch = torch_module()
    if hasattr(a, "is_cuda") and a.is_cuda:
        return a.detach().to(torch.float32).contiguous()
    return torch.as_tensor(np.ascontiguousarray(to_numpy(a), dtype=np.float32),
                           device=cuda_device())


def noll_to_zernike(j: int) -> Tuple[int, int]:
    """``(n, m)`` of Noll index ``j >= 1``: radial order n, signed azimuthal
    order m (cosine terms even j, sine terms odd j, Noll 1976)."""
    if j < 1:
        raise ValueError("Noll index j must be >= 1")
    n = int(np.floor((np.sqrt(8 * j - 7) - 1) / 2))   # j lies in row n of the triangle
    k = j - n * (n + 1) // 2                            # 1-based position within row n
    # |m| runs n % 2, n % 2 (+2 each pair) ... through the row
    am = (n % 2) + 2 * ((k - 1 + (1 - n % 2)) // 2)
    return n, (am if j % 2 == 0 or am == 0 else -am)


def _radial(n: int, am: int, rho: np.ndarray) -> np.ndarray:
    out = np.zeros_like(rho)
    for s in range((n - am) // 2 + 1):
        c = (-1) ** s * factorial(n - s) / (factorial(s) * factorial((n + am) // 2 - s)
                                            * factorial((n - am) // 2 - s))
        out += c * rho ** (n - 2 * s)
    return out


def zernike_basis(n_modes: int, n_pixels: int,
                  diameter_pixels: Optional[float] = None) -> np.ndarray:
    """``(n_modes, n_pixels, n_pixels)`` Noll-ordered Zernike modes on the
    inscribed disc (radius ``diameter_pixels / 2``, default ``n_pixels / 2``),
    unit variance over the pupil, zero outside; axis 0 is x."""
    if n_modes < 1 or n_pixels < 2:
        raise ValueError("n_modes >= 1 and n_pixels >= 2 required")
    radius = (n_pixels if diameter_pixels is None else diameter_pixels) / 2.0
    u = (np.arange(n_pixels) - (n_pixels - 1) / 2.0) / radius
    x, y = np.meshgrid(u, u, indexing="ij")
    rho, theta = np.hypot(x, y), np.arctan2(y, x)
    inside = rho <= 1.0
    out = np.zeros((n_modes, n_pixels, n_pixels))
    for q in range(n_modes):
        n, m = noll_to_zernike(q + 1)
        am = abs(m)
        ang = np.cos(am * theta) if m >= 0 else np.sin(am * theta)
        norm = np.sqrt(n + 1.0) * (np.sqrt(2.0) if m != 0 else 1.0)
        out[q] = np.where(inside, norm * _radial(n, am, rho) * ang, 0.0)
    return out


@lru_cache(maxsize=8)
def _projector(n_modes: int, n_pixels: int, diameter: Optional[float]):
    basis = zernike_basis(n_modes, n_pixels, diameter)
    return _projector_from(basis)


def _projector_from(basis: np.ndarray):
    """Pseudo-inverse of the pupil design matrix, scattered back onto the full
    grid: ``(n_modes, n_pixels^2)`` float32 on the device."""
    torch = torch_module()
    mask = basis[0] != 0
    design = basis[:, mask].T                       # (n_pupil, n_modes)
    pinv = np.linalg.pinv(design)                   # (n_modes, n_pupil), FP64
    full = np.zeros((basis.shape[0], mask.size))
    full[:, mask.ravel()] = pinv
    return torch.as_tensor(full.astype(np.float32), device=cuda_device())


def zernike_decompose(phase, n_modes: int, basis: Optional[np.ndarray] = None) -> np.ndarray:
    """Least-squares Noll coefficients ``(n_modes,)`` of an ``(n, n)`` screen or
    ``(count, n_modes)`` of a stack, in the phase's units (device GEMM)."""
    torch = torch_module()
    x = _device_f32(phase)
    single = x.dim() == 2
    if single:
        x = x[None]
    count, n = x.shape[0], x.shape[-1]
    P = _projector(int(n_modes), int(n), None) if basis is None else _projector_from(
        np.asarray(basis, dtype=np.float64))
    R, K = P.shape
    if K != n * x.shape[-2]:
        raise ValueError("basis does not match the screen size")
    lib = _lib.load()
    work = torch.empty(int(lib.pt_matmul_nt_workspace_bytes(R, K, count)), dtype=torch.uint8,
                       device=x.device)
    out = torch.empty((count, R), dtype=torch.float32, device=x.device)
    _lib.call("pt_matmul_nt", R, K, count, dptr(P), dptr(x.reshape(count, K)), dptr(out),
              dptr(work), work.numel(), stream_handle())
    c = out.double().cpu().numpy()
    return c[0] if single else c


def structure_function(phase, pixel_scale: float = 1.0,
                       max_separation: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray]:
    """``(r, D)``: separations ``1..max_separation`` (default ``n // 4``) times
    ``pixel_scale`` and the phase structure function averaged over both axes
    and the stack, ``D(r) = <[phi(x) - phi(x + r)]^2>``."""
    torch = torch_module()
    x = _device_f32(phase)
    if x.dim() == 2:
        x = x[None]
    count, ny, nx = x.shape
    n = min(ny, nx)
    ms = n // 4 if max_separation is None else int(max_separation)
    if not 1 <= ms < n:
        raise ValueError("max_separation must be in [1, n)")
    lib = _lib.load()
    work = torch.empty(int(lib.pt_structure_workspace_bytes(count, ny, nx, ms)),
                       dtype=torch.uint8, device=x.device)
    D = torch.empty(ms, dtype=torch.float64, device=x.device)
    _lib.call("pt_structure_function", count, ny, nx, dptr(x), ms, dptr(D), dptr(work),
              work.numel(), stream_handle())
    return np.arange(1, ms + 1) * float(pixel_scale), D.cpu().numpy()


@lru_cache(maxsize=8)
def _psd_grid(T: int):
    from .fourier import Grid

    return Grid(T, 1.0, np.zeros((0, 3)), workspace=False)


def temporal_psd(series, dt: float) -> Tuple[np.ndarray, np.ndarray]:
    """``(freq, psd)``: positive frequencies [Hz] (no DC) and the one-sided
    PSD of the series (samples along the last axis; other axes are averaged),
    scaled so that ``sum(psd) * df`` approximates the variance."""
    torch = torch_module()
    if not dt > 0:
        raise ValueError("dt must be positive")
    x = _device_f32(series)
    T = int(x.shape[-1])
    if T < 2:
        raise ValueError("need at least two samples")
    x = x.reshape(-1, T).contiguous()
    count = int(x.shape[0])
    grid = _psd_grid(T)
    lib = _lib.load()
    work = torch.empty(int(lib.pt_temporal_psd_workspace_bytes(grid.handle, count)),
                       dtype=torch.uint8, device=x.device)
    psd = torch.empty(T // 2 + 1, dtype=torch.float32, device=x.device)
    _lib.call("pt_temporal_psd", grid.handle, count, dptr(x), float(dt), dptr(psd), dptr(work),
              work.numel(), stream_handle())
    freq = np.fft.rfftfreq(T, d=dt)
    return freq[1:], psd.double().cpu().numpy()[1:]
