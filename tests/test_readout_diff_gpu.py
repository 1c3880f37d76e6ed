"""Differentiable readout kernels against the float64 oracle (forward and
vector-Jacobian product), determinism, edge cases and a small Adam fit."""

import numpy as np
import pytest

from oracle import readout_diff as rd

pytestmark = pytest.mark.gpu

TOL_FWD = 1e-5   # relative L2, float32 kernel vs float64 oracle
TOL_GRAD = 1e-4  # relative L2 of each gradient


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_case(seed, B, L, S, T, D, n, lgs_mag=None, spread=300.0):
    rng = np.random.default_rng(seed)
    screens = rng.standard_normal((B, L, S, S)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, L).astype(np.float32)
    mag = np.ones((D, L))
    if lgs_mag is not None:
        mag[-1] = lgs_mag
    pos0 = rng.uniform(-spread, spread, (T, D, L, 2))
    pos0[0, 0, 0] = [S - 0.25, -0.6]   # samples across the periodic seam
    g = rng.standard_normal((B, T, D, n, n)).astype(np.float32)
    return screens, w, pos0, mag, n, g


def run_gpu(screens, w, pos0, mag, n, g):
    import torch

    from pyturb_gb300.diff import layer_readout

    dev = torch.device("cuda")
    ts = torch.tensor(screens, device=dev, requires_grad=True)
    tw = torch.tensor(w, device=dev, requires_grad=True)
    tp = torch.tensor(pos0, device=dev, requires_grad=True)
    out = layer_readout(ts, tw, tp, mag, n)
    out.backward(torch.tensor(g, device=dev))
    torch.cuda.synchronize()
    return (out.detach().cpu().numpy(), ts.grad.cpu().numpy(), tw.grad.cpu().numpy(),
            tp.grad.cpu().numpy())


CASES = [
    # seed, B, L, S, T, D, n, lgs magnifications of the last direction
    (1, 2, 3, 96, 3, 3, 40, [1.0, 0.85, 0.7]),
    (2, 1, 4, 130, 2, 2, 70, [0.95, 0.9, 0.8, 0.6]),      # partial tiles, ragged bands
    (3, 2, 1, 64, 2, 1, 61, None),                          # S = one tile, n near S
    (4, 1, 9, 200, 2, 4, 129, list(np.linspace(1.0, 0.78, 9))),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"S{c[3]}_n{c[6]}_L{c[2]}")
def test_forward_and_vjp_match_oracle(case):
    seed, B, L, S, T, D, n, lm = case
    screens, w, pos0, mag, n, g = make_case(seed, B, L, S, T, D, n, lm)
    out, gs, gw, gp = run_gpu(screens, w, pos0, mag, n, g)
    ref = rd.layer_readout(screens.astype(np.float64), w.astype(np.float64), pos0, mag, n)
    assert rel(out, ref) < TOL_FWD
    rgs, rgw, rgp = rd.layer_readout_vjp(screens, w.astype(np.float64), pos0, mag, n, g)
    assert rel(gs, rgs) < TOL_GRAD
    assert rel(gw, rgw) < TOL_GRAD
    assert rel(gp, rgp) < TOL_GRAD


def test_far_positions_wrap_exactly():
    # positions millions of pixels away read the same samples as their residues mod S
    screens, w, pos0, mag, n, g = make_case(7, 1, 2, 96, 2, 2, 32)
    S = 96
    pos0 = np.round(pos0 * 2.0 ** 20) / 2.0 ** 20   # exact after adding whole periods
    far = pos0 + S * np.array([31250.0, -41667.0])
    a = run_gpu(screens, w, pos0, mag, n, g)
    b = run_gpu(screens, w, far, mag, n, g)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_backward_is_deterministic():
    screens, w, pos0, mag, n, g = make_case(8, 2, 3, 128, 4, 3, 64, [1.0, 0.9, 0.75])
    a = run_gpu(screens, w, pos0, mag, n, g)
    b = run_gpu(screens, w, pos0, mag, n, g)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_argument_errors():
    import torch

    from pyturb_gb300.diff import layer_readout

    dev = torch.device("cuda")
    s = torch.zeros((1, 2, 64, 64), device=dev)
    w = torch.ones(2, device=dev)
    p = torch.zeros((1, 1, 2, 2), dtype=torch.float64, device=dev)
    with pytest.raises(ValueError):
        layer_readout(s, w, p, np.full((1, 2), 0.1), 16)      # magnification below 0.25
    with pytest.raises(ValueError):
        layer_readout(s, w, p, np.ones((1, 2)), 64)           # footprint not smaller than S
    with pytest.raises(ValueError):
        layer_readout(s.double(), w, p, np.ones((1, 2)), 16)  # float64 screens


def test_physical_readout_and_adam_fit_recover_winds_and_weights():
    import torch

    from pyturb_gb300.diff import DifferentiableReadout, fit_layers

    rng = np.random.default_rng(11)
    L, n, S, dx = 3, 48, 96, 0.05
    alts = np.array([0.0, 4000.0, 10000.0])
    dirs = np.array([[0.0, 0.0], [2e-5, -1e-5], [0.0, 0.0]])
    times = np.arange(6) * 2e-3
    ro = DifferentiableReadout(n, S, dx, alts, dirs, times,
                               source_altitudes=[None, None, 90000.0])
    # smooth screens so that the loss is smooth in the winds
    k = np.fft.fftfreq(S)
    filt = np.exp(-(k[:, None] ** 2 + k[None, :] ** 2) / (2 * 0.03 ** 2))
    scr = np.real(np.fft.ifft2(np.fft.fft2(rng.standard_normal((1, L, S, S))) * filt))
    scr = (scr / scr.std()).astype(np.float32)
    dev = torch.device("cuda")
    screens = torch.tensor(scr, device=dev)
    w_true = torch.tensor([0.8, 0.5, 0.3], device=dev)
    v_true = torch.tensor([[5.0, -3.0], [12.0, 4.0], [-8.0, 9.0]], dtype=torch.float64, device=dev)
    target = ro(screens, w_true, v_true).detach()
    w0 = w_true * torch.tensor([1.2, 0.8, 1.25], device=dev)
    v0 = v_true + torch.tensor([[1.0, -1.0], [-1.5, 1.0], [1.0, 1.5]], dtype=torch.float64,
                               device=dev)
    w, v, losses = fit_layers(ro, screens, target, w0, v0, steps=300, lr=0.05)
    assert losses[-1] < 1e-3 * losses[0]
    np.testing.assert_allclose(w.cpu().numpy(), w_true.cpu().numpy(), rtol=0.02)
    np.testing.assert_allclose(v.cpu().numpy(), v_true.cpu().numpy(), atol=0.25)


def test_checkpointed_readout_loss_matches_the_materialised_one():
    """readout_mse (frames recomputed 3 time steps at a time) equals torch's MSE
    of the materialised frames: value and the screen, weight and wind gradients."""
    import torch

    from pyturb_gb300.diff import DifferentiableReadout

    rng = np.random.default_rng(13)
    B, L, S, n, T = 2, 3, 96, 40, 7
    dirs = [[0.0, 0.0], [2e-5, -1e-5]]
    ro = DifferentiableReadout(n, S, 0.02, [0.0, 4000.0, 9000.0], dirs, np.arange(T) * 1e-3,
                               source_altitudes=[None, 90e3])
    dev = torch.device("cuda")
    s0 = torch.tensor(rng.standard_normal((B, L, S, S)), dtype=torch.float32, device=dev)
    w0 = torch.tensor([0.9, 0.6, 0.4], device=dev)
    v0 = torch.tensor([[5.0, 1.0], [-8.0, 4.0], [12.0, -3.0]], dtype=torch.float64, device=dev)
    with torch.no_grad():
        target = ro(s0, w0 * 1.2, v0 + 1.0)
    grads = []
    for mode in ("materialised", "checkpointed"):
        sc = s0.clone().requires_grad_(True)
        w = w0.clone().requires_grad_(True)
        v = v0.clone().requires_grad_(True)
        if mode == "materialised":
            loss = torch.nn.functional.mse_loss(ro(sc, w, v), target)
        else:
            loss = ro.mse(sc, w, v, target, frames_per_chunk=3)
        loss.backward()
        grads.append([loss.detach(), sc.grad, w.grad, v.grad])
    for a, b in zip(*grads):
        a, b = a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(a)



def test_config4_geometry_matches_oracle():
    """The benchmark geometry at full size for one batch element and two
    frames: 9 layers of 768^2, 8 NGS directions in a 60" disc + 1 LGS at
    90 km, pupil 512^2, frozen-flow winds; forward and every gradient against
    the float64 oracle."""
    rng = np.random.default_rng(44)
    L, S, n, T = 9, 768, 512, 2
    heights = np.array([0.0, 500.0, 1000.0, 2000.0, 4000.0, 6000.0, 8000.0, 12000.0, 16000.0])
    rad = np.deg2rad(60.0 / 3600.0) * np.sqrt(rng.uniform(0, 1, 8))
    ang = rng.uniform(0, 2 * np.pi, 8)
    dirs = np.concatenate([np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1), [[0.0, 0.0]]])
    D = dirs.shape[0]
    mag = np.ones((D, L))
    mag[-1] = 1.0 - heights / 90e3
    winds = rng.uniform(-25, 25, (L, 2))
    dx = 8.0 / n
    pos0 = rd.positions(n, S, dx, heights, dirs, mag, winds, np.arange(T) * 1e-3)
    screens = rng.standard_normal((1, L, S, S)).astype(np.float32)
    w = rng.uniform(0.2, 0.6, L).astype(np.float32)
    g = rng.standard_normal((1, T, D, n, n)).astype(np.float32)
    out, gs, gw, gp = run_gpu(screens, w, pos0, mag, n, g)
    ref = rd.layer_readout(screens.astype(np.float64), w.astype(np.float64), pos0, mag, n)
    rgs, rgw, rgp = rd.layer_readout_vjp(screens, w.astype(np.float64), pos0, mag, n, g)
    errs = [rel(out, ref), rel(gs, rgs), rel(gw, rgw), rel(gp, rgp)]
    print("config-4 geometry rel-L2: forward %.2e, screens %.2e, weights %.2e, positions %.2e"
          % tuple(errs))
    assert errs[0] < TOL_FWD
    assert max(errs[1:]) < TOL_GRAD
