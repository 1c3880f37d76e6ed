"""The float64 synthesis oracle's VJP against central differences and torch
autograd (CPU)."""

import numpy as np
import pytest

from oracle import synth_diff as sd


def case(seed=4, L=3, ns=16, F=3, crop=2, n_out=11):
    rng = np.random.default_rng(seed)
    S = rng.standard_normal((L, ns, ns)) + 1j * rng.standard_normal((L, ns, ns))
    w = rng.uniform(0.5, 1.5, L)
    dx = 0.1
    sx = rng.uniform(-3, 3, (F, L))
    sy = rng.uniform(-3, 3, (F, L))
    g = rng.standard_normal((F, n_out, n_out))
    return S, w, sx, sy, dx, crop, n_out, 0.7, g


def value(S, w, sx, sy, dx, crop, n_out, scale, g):
    return float(np.sum(sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale) * g))


def test_vjp_matches_central_differences():
    S, w, sx, sy, dx, crop, n_out, scale, g = case()
    gS, gw, gsx, gsy = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g)
    eps = 1e-6
    args = (dx, crop, n_out, scale, g)
    for idx in [(0, 1, 2), (2, 15, 0), (1, 8, 8)]:
        for part, unit in (("re", 1.0), ("im", 1j)):
            Sp, Sm = S.copy(), S.copy()
            Sp[idx] += eps * unit
            Sm[idx] -= eps * unit
            fd = (value(Sp, w, sx, sy, *args) - value(Sm, w, sx, sy, *args)) / (2 * eps)
            want = gS[idx].real if part == "re" else gS[idx].imag
            assert fd == pytest.approx(want, rel=1e-6, abs=1e-7)
    for l in range(w.size):
        wp, wm = w.copy(), w.copy()
        wp[l] += eps
        wm[l] -= eps
        fd = (value(S, wp, sx, sy, *args) - value(S, wm, sx, sy, *args)) / (2 * eps)
        assert fd == pytest.approx(gw[l], rel=1e-6)
    for idx in [(0, 0), (2, 1), (1, 2)]:
        for arr, gref in ((sx, gsx), (sy, gsy)):
            ap, am = arr.copy(), arr.copy()
            ap[idx] += eps
            am[idx] -= eps
            if arr is sx:
                fd = (value(S, w, ap, sy, *args) - value(S, w, am, sy, *args)) / (2 * eps)
            else:
                fd = (value(S, w, sx, ap, *args) - value(S, w, sx, am, *args)) / (2 * eps)
            assert fd == pytest.approx(gref[idx], rel=1e-5, abs=1e-6)


def test_vjp_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    S, w, sx, sy, dx, crop, n_out, scale, g = case(seed=9)
    L, ns, _ = S.shape
    tS = torch.tensor(S, requires_grad=True)
    tw = torch.tensor(w, requires_grad=True)
    tsx = torch.tensor(sx, requires_grad=True)
    tsy = torch.tensor(sy, requires_grad=True)
    f = torch.tensor(np.fft.fftfreq(ns, dx))
    px = torch.exp(2j * np.pi * f[None, None, :] * tsx[..., None])
    py = torch.exp(2j * np.pi * f[None, None, :] * tsy[..., None])
    X = torch.einsum("l,lij,fli,flj->fij", tw.to(torch.complex128), tS, px, py)
    y = scale * torch.fft.ifft2(X).real * ns * ns
    y = y[:, crop:crop + n_out, crop:crop + n_out]
    (y * torch.tensor(g)).sum().backward()
    gS, gw, gsx, gsy = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g)
    np.testing.assert_allclose(y.detach().numpy(),
                               sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale),
                               rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(tS.grad.numpy(), gS, rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(tw.grad.numpy(), gw, rtol=1e-10)
    np.testing.assert_allclose(tsx.grad.numpy(), gsx, rtol=1e-9, atol=1e-8)
    np.testing.assert_allclose(tsy.grad.numpy(), gsy, rtol=1e-9, atol=1e-8)


def sh_case(seed=6, L=2, ns=18, F=3, P=2):
    rng = np.random.default_rng(seed)
    coef = rng.standard_normal((P, L, 3, 3)) + 1j * rng.standard_normal((P, L, 3, 3))
    dx = 0.1
    df = 1.0 / (ns * dx)
    freqs = np.array([[-1.0, 0.0, 1.0]]) * df / 3.0 ** np.arange(1, P + 1)[:, None]
    return coef, freqs


def test_subharmonic_forward_follows_the_reference_layout():
    # low = Re(basis^T (shifted @ basis)) - mean, shifted = sum_l c px py (atmosphere.py:921-935)
    S, w, sx, sy, dx, crop, n_out, scale, g = case(seed=3)
    coef, freqs = sh_case(L=S.shape[0], ns=S.shape[-1])
    ns = S.shape[-1]
    with_sh = sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale, sh=(coef, freqs))
    without = sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale)
    x = (np.arange(ns) - ns / 2.0) * dx
    basis = np.exp(2j * np.pi * freqs[:, :, None] * x[None, None, :])
    for f in range(sx.shape[0]):
        px = np.exp(2j * np.pi * sx[f][None, :, None] * freqs[:, None, :])
        py = np.exp(2j * np.pi * sy[f][None, :, None] * freqs[:, None, :])
        shifted = ((coef * w[None, :, None, None]) * px[:, :, :, None] * py[:, :, None, :]).sum(1)
        m = np.matmul(shifted, basis).reshape(-1, ns)
        low = (basis.reshape(-1, ns).T @ m).real
        low -= low.mean()
        np.testing.assert_allclose(with_sh[f] - without[f],
                                   scale * low[crop:crop + n_out, crop:crop + n_out],
                                   rtol=1e-10, atol=1e-12)


def test_subharmonic_vjp_matches_central_differences():
    S, w, sx, sy, dx, crop, n_out, scale, g = case(seed=8, L=2, ns=18, n_out=13)
    coef, freqs = sh_case(L=2)
    sh = (coef, freqs)
    gS, gw, gsx, gsy, gc = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g, sh=sh)

    def val(w_=w, sx_=sx, sy_=sy, c_=coef):
        return float(np.sum(sd.synth_frames(S, w_, sx_, sy_, dx, crop, n_out, scale,
                                            sh=(c_, freqs)) * g))

    eps = 1e-6
    for l in range(w.size):
        wp, wm = w.copy(), w.copy()
        wp[l] += eps
        wm[l] -= eps
        assert (val(w_=wp) - val(w_=wm)) / (2 * eps) == pytest.approx(gw[l], rel=1e-6)
    for idx in [(0, 0), (2, 1), (1, 0)]:
        for name, arr, gref in (("x", sx, gsx), ("y", sy, gsy)):
            ap, am = arr.copy(), arr.copy()
            ap[idx] += eps
            am[idx] -= eps
            kw = "sx_" if name == "x" else "sy_"
            fd = (val(**{kw: ap}) - val(**{kw: am})) / (2 * eps)
            assert fd == pytest.approx(gref[idx], rel=1e-5, abs=1e-6)
    for idx in [(0, 0, 0, 1), (1, 1, 2, 2), (0, 1, 1, 0)]:
        for part, unit in (("re", 1.0), ("im", 1j)):
            cp, cm = coef.copy(), coef.copy()
            cp[idx] += eps * unit
            cm[idx] -= eps * unit
            fd = (val(c_=cp) - val(c_=cm)) / (2 * eps)
            want = gc[idx].real if part == "re" else gc[idx].imag
            assert fd == pytest.approx(want, rel=1e-6, abs=1e-7)


def test_subharmonic_vjp_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    S, w, sx, sy, dx, crop, n_out, scale, g = case(seed=12, L=2, ns=16, n_out=11)
    coef, freqs = sh_case(L=2, ns=16)
    L, ns, _ = S.shape
    tS = torch.tensor(S, requires_grad=True)
    tw = torch.tensor(w, requires_grad=True)
    tsx = torch.tensor(sx, requires_grad=True)
    tsy = torch.tensor(sy, requires_grad=True)
    tc = torch.tensor(coef, requires_grad=True)
    f = torch.tensor(np.fft.fftfreq(ns, dx))
    fp = torch.tensor(freqs)
    px = torch.exp(2j * np.pi * f[None, None, :] * tsx[..., None])
    py = torch.exp(2j * np.pi * f[None, None, :] * tsy[..., None])
    X = torch.einsum("l,lij,fli,flj->fij", tw.to(torch.complex128), tS, px, py)
    y = torch.fft.ifft2(X).real * ns * ns
    x = torch.tensor((np.arange(ns) - ns / 2.0) * dx)
    basis = torch.exp(2j * np.pi * fp[:, :, None] * x[None, None, :])           # (P, 3, ns)
    ex = torch.exp(2j * np.pi * tsx[:, :, None, None] * fp[None, None])          # (F, L, P, 3)
    ey = torch.exp(2j * np.pi * tsy[:, :, None, None] * fp[None, None])
    C = torch.einsum("l,plij,flpi,flpj->fpij", tw.to(torch.complex128), tc, ex, ey)
    low = torch.einsum("pix,fpij,pjy->fxy", basis, C, basis).real
    y = y + low - low.mean(dim=(1, 2), keepdim=True)
    y = scale * y[:, crop:crop + n_out, crop:crop + n_out]
    (y * torch.tensor(g)).sum().backward()
    gS, gw, gsx, gsy, gc = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g, sh=(coef, freqs))
    np.testing.assert_allclose(y.detach().numpy(),
                               sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale,
                                               sh=(coef, freqs)), rtol=1e-11, atol=1e-10)
    np.testing.assert_allclose(tS.grad.numpy(), gS, rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(tw.grad.numpy(), gw, rtol=1e-10)
    np.testing.assert_allclose(tsx.grad.numpy(), gsx, rtol=1e-9, atol=1e-8)
    np.testing.assert_allclose(tsy.grad.numpy(), gsy, rtol=1e-9, atol=1e-8)
    np.testing.assert_allclose(tc.grad.numpy(), gc, rtol=1e-10, atol=1e-10)
