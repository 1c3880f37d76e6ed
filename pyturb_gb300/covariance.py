"""The Assemat-Wilson extrusion operator, built on the GPU in FP64.

``build_operator`` replaces the reference's host recipe (covariances with
``scipy.special.kv``, Cholesky solve, eigen square root:
``src/pyturb/infinite.py:54-117``, ``src/pyturb/extrude.py:250-304``) by one
native call, ``pt_aw_build``: the joint von Karman covariance of the stencil
and the new row is factored once on the device, which yields ``A``, a factor
``B`` of the conditional covariance and the stencil factor ``S`` together.

``B`` is not unique. The default is the Cholesky factor the build produces.
``b_factor="eigh"`` instead takes the eigen square root of the same
conditional covariance (the factor the reference uses), so that noise drawn
in the reference's order reproduces the reference's screens: the parity mode.

The stencil is ``m`` full rows, optionally extended by sparse points
(``sparse_points``): columns evenly spaced across the row, at depths
4, 8, 16, ... rows behind the new row. The reference has only the full rows;
the sparse points carry the large-scale, along-wind correlation that two rows
cannot.
"""

from __future__ import annotations

import ctypes as C
import math
import warnings
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .backend import cuda_device, dptr, stream_handle, torch_module

__all__ = ["phase_covariance", "build_operator", "build_extrusion", "seed_factor",
           "sparse_points", "ExtrusionOperator", "AnchorTables", "dct_modes", "anchor_modes"]

_NU = 5.0 / 6.0


def _vk_prefactor(r0: float, L0: float) -> float:
    """``(L0/r0)^{5/3} 2^{-5/6} Gamma(11/6) / pi^{8/3} ((24/5) Gamma(6/5))^{5/6}``."""
    return ((L0 / r0) ** (5.0 / 3.0) * 2.0 ** (-5.0 / 6.0) * math.gamma(11.0 / 6.0)
            / math.pi ** (8.0 / 3.0) * (4.8 * math.gamma(1.2)) ** (5.0 / 6.0))


def _x_nu_k_nu(x: np.ndarray) -> np.ndarray:
    """``x^{5/6} K_{5/6}(x)`` for x > 0 by the trapezoidal rule on
    ``K_nu(x) = int_0^inf exp(-x cosh t) cosh(nu t) dt`` (geometric
    convergence: the integrand is analytic in |Im t| < pi/2), the same
    evaluation the device build uses."""
    out = np.zeros_like(x)
    live = np.flatnonzero((x > 0) & (x <= 700.0))
    if live.size == 0:
        return out
    xv = x[live]
    h = np.minimum(0.25, 0.7 / np.sqrt(xv))
    total = 0.5 * np.exp(-xv)
    todo = np.arange(xv.size)
    k = 1
    while todo.size and k < 4096:
        t = k * h[todo]
        term = np.exp(-xv[todo] * np.cosh(t)) * np.cosh(_NU * t)
        total[todo] += term
        todo = todo[term >= 1e-18 * total[todo]]
        k += 1
    out[live] = xv ** _NU * h * total
    return out


def phase_covariance(r, r0: float, L0: float) -> np.ndarray:
    """Von Karman phase covariance [rad^2] at separations ``r`` [m]
    (``pyturb.infinite.phase_covariance``, ``src/pyturb/infinite.py:88-117``):
    ``C(r) = c x^{5/6} K_{5/6}(x)``, ``x = 2 pi r / L0``, and
    ``c 2^{-1/6} Gamma(5/6)`` at r = 0."""
    if not np.isfinite(L0):
        raise ValueError("phase_covariance requires a finite outer scale L0")
    r = np.asarray(r, dtype=np.float64)
    x = (2.0 * np.pi / L0) * r
    core = _x_nu_k_nu(np.atleast_1d(x).ravel()).reshape(x.shape)
    core = np.where(x > 0, core, 2.0 ** (-1.0 / 6.0) * math.gamma(_NU))
    return _vk_prefactor(r0, L0) * core


def sparse_points(width: int, stencil_rows: int, columns: int,
                  max_depth: Optional[int] = None) -> List[Tuple[int, int]]:
    """Sparse stencil points ``(depth, column)``: ``columns`` columns at
    ``round((c + 1) (W - 1) / (columns + 1))``, each at every depth 2^j with
    ``stencil_rows < 2^j <= max_depth`` (default: the largest power of two
    not above the width)."""
    W, m, k = int(width), int(stencil_rows), int(columns)
    if k <= 0:
        return []
    dmax = int(max_depth) if max_depth is not None else 1 << (W.bit_length() - 1)
    depths = []
    d = 2
    while d <= dmax:
        if d > m:
            depths.append(d)
        d *= 2
    cols = [int(round((c + 1) * (W - 1) / (k + 1))) for c in range(k)]
    pts = [(d, c) for d in depths for c in cols]
    if len(pts) > _lib.PT_MAX_SPARSE:
        raise ValueError(f"{len(pts)} sparse stencil points; at most {_lib.PT_MAX_SPARSE}")
    return pts


class ExtrusionOperator:
    """Device operator of one outer scale: ``M = [A | B]`` float32 ``(W, K)``
    (``K = (m + 1) W + len(sparse)``), optionally its float64 twin ``M64``,
    the float32 rounding of the stencil part ``Mlo = A - float32(A)``
    (``(W, Kz)``, ``Kz = m W + len(sparse)``) and the stencil factor ``S``
    (float32 ``(Kz, Kz)``, ``S S^T = C_zz``), all at unit r0."""

    def __init__(self, W: int, m: int, sparse, M, M64=None, S=None, Mlo=None,
                 increments: bool = False):
        self.W, self.m = int(W), int(m)
        self.sparse = list(sparse)
        self.Kz = self.m * self.W + len(self.sparse)
        self.M, self.M64, self.S, self.Mlo = M, M64, S, Mlo
        self.increments = bool(increments)

    def host(self, r0: float = 1.0) -> Tuple[np.ndarray, np.ndarray]:
        """``(A, B)`` as float64 host arrays, ``B`` scaled by r0^(-5/6)."""
        src = self.M64 if self.M64 is not None else self.M
        full = src.double().cpu().numpy()
        return full[:, :self.Kz].copy(), full[:, self.Kz:] * float(r0) ** (-5.0 / 6.0)


def build_operator(width: int, stencil_rows: int, pixel_scale: float, L0: float,
                   sparse: Sequence[Tuple[int, int]] = (), b_factor: str = "cholesky",
                   want_seed: bool = False, want_float64: bool = False,
                   want_lo: bool = False, increments: bool = False) -> ExtrusionOperator:
    """Build ``[A | B]`` for extruding one ``width``-pixel row from the stencil
    (``stencil_rows`` full rows below it, then the ``sparse`` points) at unit
    r0, in FP64 on the GPU. ``b_factor``: ``"cholesky"`` (the build's own
    factor) or ``"eigh"`` (eigen square root of the same conditional
    covariance, the reference's choice). A stencil covariance that is not
    numerically positive definite is retried with a growing diagonal load
    (1e-12 ... 1e-8 of the variance), with a warning. ``increments`` returns
    the stencil part in increment form (row differences and the newest row;
    the new row is the newest stencil row plus the product), which keeps a
    float32 recursion on the float64 one over long runs."""
    if b_factor not in ("cholesky", "eigh"):
        raise ValueError("b_factor must be 'cholesky' or 'eigh'")
    if not np.isfinite(L0):
        raise ValueError("the extrusion operator requires a finite outer scale L0")
    torch = torch_module()
    lib = _lib.load()
    W, m = int(width), int(stencil_rows)
    st = _lib.sparse_stencil(sparse)
    sp = C.byref(st) if st is not None else None
    nbytes = int(lib.pt_aw_workspace_bytes(W, m, sp))
    if nbytes == 0:
        raise ValueError("build_operator: bad width, stencil rows or sparse points")
    npts = len(list(sparse))
    K, Kz = (m + 1) * W + npts, m * W + npts
    dev = cuda_device()
    work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    M = torch.empty((W, K), dtype=torch.float32, device=dev)
    M64 = torch.empty((W, K), dtype=torch.float64, device=dev) if want_float64 else None
    S = torch.empty((Kz, Kz), dtype=torch.float32, device=dev) if want_seed else None
    Mlo = torch.empty((W, Kz), dtype=torch.float32, device=dev) if want_lo else None
    sigma = torch.empty((W, W), dtype=torch.float64, device=dev) if b_factor == "eigh" else None
    for jitter in (0.0, 1e-12, 1e-10, 1e-8):
        rc = lib.pt_aw_build(W, m, sp, float(pixel_scale), float(L0), jitter, int(increments),
                             dptr(M), dptr(M64), dptr(Mlo), dptr(S), dptr(sigma), dptr(work),
                             nbytes, stream_handle())
        if rc == _lib.PT_OK:
            break
        if rc != _lib.PT_ERR_NUMERIC or jitter == 1e-8:
            raise (ValueError if rc == _lib.PT_ERR_ARG else RuntimeError)(
                f"pt_aw_build (status {rc}): {lib.pt_last_error().decode(errors='replace')}")
        warnings.warn(f"extrusion stencil covariance is not numerically positive definite "
                      f"(W={W}, L0={L0}); retrying with a diagonal load", RuntimeWarning)
    del work
    if sigma is not None:
        cov = sigma.cpu().numpy()
        vals, vecs = np.linalg.eigh(0.5 * (cov + cov.T))
        root = vecs * np.sqrt(np.maximum(vals, 0.0))
        M[:, Kz:] = torch.from_numpy(root).to(device=dev, dtype=torch.float32)
        if M64 is not None:
            M64[:, Kz:] = torch.from_numpy(root).to(device=dev)
    return ExtrusionOperator(W, m, sparse, M, M64, S, Mlo, increments)


ANCHOR_MODES = 32


def dct_modes(width: int, modes: int = ANCHOR_MODES) -> np.ndarray:
    """Orthonormal DCT-II basis ``(modes, W)``: ``sqrt((2 - [i=0]) / W)
    cos(pi i (w + 1/2) / W)``, the smooth modes of a row."""
    w = (np.arange(width) + 0.5) / width
    U = np.cos(np.pi * np.arange(modes)[:, None] * w[None, :]) * np.sqrt(2.0 / width)
    U[0] *= np.sqrt(0.5)
    return U


def pair_order(modes: int) -> np.ndarray:
    """Mode order of an anchor table row: pairs (i, i + 16) of each block of 32."""
    return np.array([b + q + 16 * h for b in range(0, modes, 32) for q in range(16)
                     for h in range(2)])


class AnchorTables:
    """Device tables of the float32 form's low-order anchor for a stack of
    operators (one per outer-scale group): the columns of
    ``[U^T A | U^T B | -U]`` as (hi, lo) float32 pairs, modes in pair order,
    and ``U`` in float32, U the first 32 (or 64) DCT-II modes."""

    def __init__(self, ops: Sequence["ExtrusionOperator"], modes: int = ANCHOR_MODES):
        if modes not in (32, 64):
            raise ValueError("the anchor takes 32 or 64 modes")
        W = ops[0].W
        if modes > W:
            raise ValueError(f"{modes} anchored modes need rows of at least {modes} pixels")
        torch = torch_module()
        dev = cuda_device()
        U = dct_modes(W, modes)
        order = pair_order(modes)
        tabs = []
        for op in ops:
            if op.M64 is None:
                raise ValueError("the anchor needs the float64 operator (want_float64=True)")
            full = op.M64.cpu().numpy()                         # (W, K) = [A | B]
            blocks = [U @ full, -U] + ([U] if op.increments else [])  # (+ r1 in increment form)
            cols = np.concatenate(blocks, axis=1)               # (modes, K + W (+ W))
            tabs.append(cols[order].T)                          # (K + W, modes)
        t = np.ascontiguousarray(np.stack(tabs))
        hi = t.astype(np.float32)
        lo = (t - hi.astype(np.float64)).astype(np.float32)
        self.t_hi = torch.from_numpy(hi).to(dev)
        self.t_lo = torch.from_numpy(lo).to(dev)
        self.u = torch.from_numpy(U.astype(np.float32)).to(dev)
        self.modes = modes
        self.struct = _lib.ExtrudeAnchor(modes=modes, pad=0, t_hi=dptr(self.t_hi),
                                         t_lo=dptr(self.t_lo), u=dptr(self.u))


def anchor_modes(width: int, sparse) -> int:
    """Anchored modes for a row of ``width`` pixels: 64 with a sparse stencil
    (its deep points give rounding errors a longer memory), 32 for full rows
    only, none below 32 pixels."""
    if width < 32:
        return 0
    return 64 if sparse and width >= 256 else 32


def build_extrusion(width: int, stencil_rows: int, pixel_scale: float, L0: float,
                    r0: float = 1.0, sparse: Sequence[Tuple[int, int]] = (),
                    b_factor: str = "eigh") -> Tuple[np.ndarray, np.ndarray]:
    """Host float64 ``(A (W, Kz), B (W, W))`` from the FP64 device build, B
    scaled by r0^(-5/6) (the return of the reference's ``build_extrusion``,
    ``src/pyturb/extrude.py:250-304``, eigen-square-root ``B`` by default)."""
    op = build_operator(width, stencil_rows, pixel_scale, L0, sparse, b_factor=b_factor,
                        want_float64=True)
    return op.host(r0)


def seed_factor(width: int, stencil_rows: int, pixel_scale: float, L0: float,
                sparse: Sequence[Tuple[int, int]] = ()):
    """Device float32 ``S`` with ``S S^T = C_zz`` (unit r0): the stencil part
    of the same factorisation, the seed of boiling's fresh windows
    (``src/pyturb/extrude.py:290-303``)."""
    return build_operator(width, stencil_rows, pixel_scale, L0, sparse, want_seed=True).S
