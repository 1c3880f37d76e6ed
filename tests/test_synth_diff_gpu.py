"""Spectral-synthesis adjoint against the float64 oracle: forward frames,
gradients for spectra, weights and shifts, and a small fit of winds."""

import numpy as np
import pytest

from oracle import synth_diff as sd

pytestmark = pytest.mark.gpu

TOL_FWD = 1e-5
TOL_GRAD = 1e-4


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run(S, w, sx, sy, dx, crop, n_out, scale, g):
    import torch

    from pyturb_gb300.diff import spectral_synthesis
    from pyturb_gb300.fourier import Grid

    ns = S.shape[-1]
    dev = torch.device("cuda")
    grid = Grid(ns, dx, np.zeros((0, 3)))
    tS = torch.tensor(S.astype(np.complex64), device=dev, requires_grad=True)
    tw = torch.tensor(w.astype(np.float32), device=dev, requires_grad=True)
    tsh = torch.tensor(np.stack([sx, sy], -1), dtype=torch.float64, device=dev, requires_grad=True)
    out = spectral_synthesis(tS, tw, tsh, grid, crop, n_out, scale)
    out.backward(torch.tensor(g.astype(np.float32), device=dev))
    torch.cuda.synchronize()
    gsh = tsh.grad.cpu().numpy()
    return (out.detach().cpu().numpy(), tS.grad.cpu().numpy(), tw.grad.cpu().numpy(),
            gsh[..., 0], gsh[..., 1])


@pytest.mark.parametrize("uniform", [False, True], ids=["arbitrary", "uniform"])
@pytest.mark.parametrize("ns,F,L", [(64, 5, 3), (96, 4, 2), (512, 6, 9), (202, 4, 2)])
def test_synthesis_and_vjp_match_oracle(ns, F, L, uniform):
    rng = np.random.default_rng(ns + F + L)
    S = (rng.standard_normal((L, ns, ns)) + 1j * rng.standard_normal((L, ns, ns))) / ns
    w = rng.uniform(0.5, 1.5, L)
    dx = 8.0 / ns
    if uniform:   # equally spaced frames take the register-recurrence path
        v = rng.uniform(-20, 20, (L, 2))
        t = np.arange(F) * 1e-3
        sx, sy = t[:, None] * v[None, :, 0], t[:, None] * v[None, :, 1]
    else:
        sx, sy = rng.uniform(-30, 30, (F, L)), rng.uniform(-30, 30, (F, L))
    crop = ns // 8
    n_out = ns - 2 * crop - 1
    scale = 0.3
    g = rng.standard_normal((F, n_out, n_out))
    out, gS, gw, gsx, gsy = run(S, w, sx, sy, dx, crop, n_out, scale, g)
    assert rel(out, sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale)) < TOL_FWD
    rS, rw, rsx, rsy = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g)
    assert rel(gS, rS) < TOL_GRAD
    assert rel(gw, rw) < TOL_GRAD
    assert rel(gsx, rsx) < TOL_GRAD
    assert rel(gsy, rsy) < TOL_GRAD


def test_subharmonic_coefficients_required_exactly_with_levels():
    import torch

    from pyturb_gb300.diff import spectral_synthesis
    from pyturb_gb300.fourier import Grid

    dev = torch.device("cuda")
    S = torch.zeros((1, 32, 32), dtype=torch.complex64, device=dev)
    sh = torch.zeros((2, 1, 2), dtype=torch.float64, device=dev)
    with pytest.raises(ValueError):   # levels on the grid, no coefficients
        spectral_synthesis(S, torch.ones(1, device=dev), sh,
                           Grid(32, 0.1, np.array([[-1.0, 0.0, 1.0]])), 0, 32)
    with pytest.raises(ValueError):   # coefficients, no levels
        spectral_synthesis(S, torch.ones(1, device=dev), sh, Grid(32, 0.1, np.zeros((0, 3))), 0,
                           32, sh_coef=torch.zeros((1, 1, 3, 3), dtype=torch.complex64,
                                                   device=dev))


def _sh_case(rng, ns, L, P, dx):
    coef = (rng.standard_normal((P, L, 3, 3)) + 1j * rng.standard_normal((P, L, 3, 3))) * 0.3
    df = 1.0 / (ns * dx)
    freqs = np.array([[-1.0, 0.0, 1.0]]) * df / 3.0 ** np.arange(1, P + 1)[:, None]
    return coef, freqs


@pytest.mark.parametrize("uniform", [False, True], ids=["arbitrary", "uniform"])
@pytest.mark.parametrize("ns,F,L,P,chunk", [(64, 5, 3, 2, 64), (128, 7, 2, 3, 3)])
def test_subharmonic_synthesis_and_vjp_match_oracle(ns, F, L, P, chunk, uniform):
    import torch

    from pyturb_gb300.diff import spectral_synthesis
    from pyturb_gb300.fourier import Grid

    rng = np.random.default_rng(ns + 7 * P)
    S = (rng.standard_normal((L, ns, ns)) + 1j * rng.standard_normal((L, ns, ns))) / ns
    w = rng.uniform(0.5, 1.5, L)
    dx = 8.0 / ns
    coef, freqs = _sh_case(rng, ns, L, P, dx)
    if uniform:
        v = rng.uniform(-20, 20, (L, 2))
        t = np.arange(F) * 1e-3
        sx, sy = t[:, None] * v[None, :, 0], t[:, None] * v[None, :, 1]
    else:
        sx, sy = rng.uniform(-30, 30, (F, L)), rng.uniform(-30, 30, (F, L))
    crop = ns // 8
    n_out = ns - 2 * crop - 1
    scale = 0.3
    g = rng.standard_normal((F, n_out, n_out))
    dev = torch.device("cuda")
    grid = Grid(ns, dx, freqs)
    tS = torch.tensor(S.astype(np.complex64), device=dev, requires_grad=True)
    tw = torch.tensor(w.astype(np.float32), device=dev, requires_grad=True)
    tsh = torch.tensor(np.stack([sx, sy], -1), dtype=torch.float64, device=dev, requires_grad=True)
    tc = torch.tensor(coef.astype(np.complex64), device=dev, requires_grad=True)
    out = spectral_synthesis(tS, tw, tsh, grid, crop, n_out, scale, sh_coef=tc,
                             frames_per_chunk=chunk)
    out.backward(torch.tensor(g.astype(np.float32), device=dev))
    torch.cuda.synchronize()
    sh = (coef, freqs)
    assert rel(out.detach().cpu().numpy(),
               sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale, sh=sh)) < TOL_FWD
    rS, rw, rsx, rsy, rc = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g, sh=sh)
    gsh = tsh.grad.cpu().numpy()
    assert rel(tS.grad.cpu().numpy(), rS) < TOL_GRAD
    assert rel(tw.grad.cpu().numpy(), rw) < TOL_GRAD
    assert rel(gsh[..., 0], rsx) < TOL_GRAD
    assert rel(gsh[..., 1], rsy) < TOL_GRAD
    assert rel(tc.grad.cpu().numpy(), rc) < TOL_GRAD


def test_checkpointed_synthesis_loss_matches_the_materialised_one():
    """The frames-recomputing MSE (chunks of 3 frames) equals torch's MSE of the
    materialised frames, value and every gradient, with subharmonic levels."""
    import torch

    from pyturb_gb300.diff import DifferentiableSpectralFrames

    rng = np.random.default_rng(21)
    L, n, ns, P = 3, 48, 64, 2
    sf = DifferentiableSpectralFrames(n, ns, 0.05, r0=0.1, L0=10.0,
                                      altitudes=[0.0, 5000.0, 10000.0],
                                      times=np.arange(5) * 2e-3,
                                      directions=[[0.0, 0.0], [1e-5, 0.0]], subharmonics=P)
    dev = torch.device("cuda")
    noise0 = torch.tensor(rng.standard_normal((L, ns, ns)) + 1j * rng.standard_normal((L, ns, ns)),
                          dtype=torch.complex64, device=dev)
    shn0 = torch.tensor(rng.standard_normal((L, P, 3, 3)) + 1j * rng.standard_normal((L, P, 3, 3)),
                        dtype=torch.complex64, device=dev)
    w0 = torch.tensor([0.8, 0.5, 0.3], device=dev)
    v0 = torch.tensor([[6.0, -2.0], [10.0, 3.0], [-7.0, 8.0]], dtype=torch.float64, device=dev)
    target = (sf(noise0, w0, v0, shn0) * 1.1).detach()
    grads = []
    for mode in ("materialised", "checkpointed"):
        noise = noise0.clone().requires_grad_(True)
        shn = shn0.clone().requires_grad_(True)
        w = (w0 * 0.9).clone().requires_grad_(True)
        v = (v0 + 0.5).clone().requires_grad_(True)
        if mode == "materialised":
            loss = torch.nn.functional.mse_loss(sf(noise, w, v, shn), target)
        else:
            loss = sf.mse(noise, w, v, target, sh_noise=shn, frames_per_chunk=3)
        loss.backward()
        grads.append([loss.detach(), noise.grad, shn.grad, w.grad, v.grad])
    for a, b in zip(*grads):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert rel(b, a) < 1e-5


def test_wind_fit_through_the_synthesis():
    import torch

    from pyturb_gb300.diff import DifferentiableSpectralFrames

    rng = np.random.default_rng(5)
    L, n, ns = 3, 48, 64
    sf = DifferentiableSpectralFrames(n, ns, 0.05, r0=0.1, L0=10.0,
                                      altitudes=[0.0, 5000.0, 10000.0],
                                      times=np.arange(8) * 2e-3,
                                      directions=[[0.0, 0.0], [1e-5, 0.0]])
    dev = torch.device("cuda")
    noise = torch.tensor(rng.standard_normal((L, ns, ns)) + 1j * rng.standard_normal((L, ns, ns)),
                         dtype=torch.complex64, device=dev)
    w_true = torch.tensor([0.8, 0.5, 0.3], device=dev)
    v_true = torch.tensor([[6.0, -2.0], [10.0, 3.0], [-7.0, 8.0]], dtype=torch.float64, device=dev)
    target = sf(noise, w_true, v_true).detach()
    w = (w_true * 1.15).clone().requires_grad_(True)
    v = (v_true + 0.8).clone().requires_grad_(True)
    opt = torch.optim.Adam([w, v], lr=0.03)
    losses = []
    for _ in range(200):
        opt.zero_grad()
        loss = torch.nn.functional.mse_loss(sf(noise, w, v), target)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < 1e-2 * losses[0]
    np.testing.assert_allclose(w.detach().cpu().numpy(), w_true.cpu().numpy(), rtol=0.05)
    np.testing.assert_allclose(v.detach().cpu().numpy(), v_true.cpu().numpy(), atol=0.5)
