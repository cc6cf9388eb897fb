"""The warm-start network's tensor-core kernels and what it gains.

The products are checked against float64 products of the same BF16
operands; the loss gradient against CPU torch float64 autograd of the same
network, with the same BF16 roundings of weights and activations (the
backward pass also rounds dZ to BF16 before its products: tolerance 2e-2
relative per parameter block, cosine above 0.999).  The trained model must
reach the mass tolerance from its learned start on a mixture it was not
trained on; the test prints the Newton iterations and cell computations
of both starts (what the network gains) and fails if the learned start
costs more than three extra Newton iterations."""
import os

import numpy as np
import pytest

from conftest import gaussian_mixture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.fixture(scope="module")
def ws():
    from geogram_gb300 import warmstart
    return warmstart


@pytest.mark.parametrize("M,N,K", [(64, 64, 32), (200, 100, 64), (1000, 128, 128), (37, 5, 96)])
def test_tensor_core_gemm(torch, ws, M, N, K):
    g = torch.Generator().manual_seed(M + N + K)
    a = torch.randn(M, K, generator=g).to(torch.bfloat16)
    bt = torch.randn(N, K, generator=g).to(torch.bfloat16)
    c = ws.gemm_nt(a.cuda(), bt.cuda()).cpu().double()
    ref = a.double() @ bt.double().T
    assert torch.max(torch.abs(c - ref)).item() <= 1e-5 * max(1.0, torch.max(torch.abs(ref)).item())


def reference_loss(torch, ws, params, norm, raw, target):
    """The network in float64 on the CPU with the kernels' BF16 roundings."""
    bf = lambda t: t.to(torch.bfloat16).double()  # noqa: E731
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    nrm = torch.tensor(norm, dtype=torch.float64)
    H, IN = ws.H, ws.IN
    W1 = p[ws.OFF_W1:ws.OFF_B1].view(H, 32)
    b1 = p[ws.OFF_B1:ws.OFF_W2]
    W2 = p[ws.OFF_W2:ws.OFF_B2].view(H, H)
    b2 = p[ws.OFF_B2:ws.OFF_W3]
    W3 = p[ws.OFF_W3:ws.OFF_B3].view(H, H)
    b3 = p[ws.OFF_B3:ws.OFF_W4]
    W4 = p[ws.OFF_W4:ws.OFF_B4]
    b4 = p[ws.OFF_B4]
    # straight-through BF16 rounding of the weights
    rw = lambda W: W + (bf(W.detach()) - W.detach())  # noqa: E731
    x = (torch.tensor(raw, dtype=torch.float64) - nrm[:IN].float().double()) / nrm[IN:2 * IN]
    x = bf(torch.cat([x, torch.zeros(x.shape[0], 32 - IN, dtype=torch.float64)], 1))
    gelu = torch.nn.functional.gelu
    h = x
    for W, b in ((W1, b1), (W2, b2), (W3, b3)):
        z = h @ rw(W).T + b
        h = gelu(z)
        h = h + (bf(h.detach()) - h.detach())
    y = h @ W4 + b4
    t = (torch.tensor(target, dtype=torch.float64) - nrm[2 * IN]) / nrm[2 * IN + 1]
    loss = ((y - t) ** 2).mean()
    loss.backward()
    return loss.item(), p.grad.numpy()


def test_gradient_vs_cpu_float64(torch, ws):
    rng = np.random.default_rng(0)
    model = ws.WarmStartModel(seed=1)
    # a model away from its initialisation: biases and scales perturbed
    model.params = model.params + rng.normal(0, 0.02, model.params.shape).astype(np.float32)
    model.params[ws.OFF_W1:ws.OFF_B1].reshape(ws.H, 32)[:, ws.IN:] = 0.0
    n = 300
    raw = rng.normal(0.5, 0.3, (n, ws.IN)).astype(np.float32)
    target = rng.normal(0.01, 0.02, n).astype(np.float32)
    norm = np.concatenate([raw.mean(0), raw.std(0), [0.01, 0.02]]).astype(np.float32)
    model.norm = norm
    model._dev = None
    loss, g = model.loss_grad(torch.tensor(raw, device="cuda"), torch.tensor(target, device="cuda"))
    g = g.cpu().numpy().astype(np.float64)
    ref_loss, ref_g = reference_loss(torch, ws, model.params, norm, raw, target)
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss
    blocks = [(ws.OFF_W1, ws.OFF_B1), (ws.OFF_B1, ws.OFF_W2), (ws.OFF_W2, ws.OFF_B2),
              (ws.OFF_B2, ws.OFF_W3), (ws.OFF_W3, ws.OFF_B3), (ws.OFF_B3, ws.OFF_W4),
              (ws.OFF_W4, ws.OFF_B4), (ws.OFF_B4, ws.OFF_B4 + 1)]
    for a, b in blocks:
        d = np.linalg.norm(g[a:b] - ref_g[a:b])
        r = np.linalg.norm(ref_g[a:b])
        assert d <= 2e-2 * r + 1e-12, (a, b, d / max(r, 1e-30))
        if b - a > 1:
            cos = g[a:b] @ ref_g[a:b] / (np.linalg.norm(g[a:b]) * r + 1e-30)
            assert cos > 0.999, (a, b, cos)
    # the padded input columns get no gradient
    assert np.all(g[ws.OFF_W1:ws.OFF_B1].reshape(ws.H, 32)[:, ws.IN:] == 0.0)


def test_training_fits_a_smooth_function(torch, ws):
    rng = np.random.default_rng(2)
    n = 20000
    raw = rng.uniform(0, 1, (n, ws.IN)).astype(np.float32)
    target = (np.sin(3 * raw[:, 0]) + raw[:, 3] * raw[:, 4] - np.cos(2 * raw[:, 10])).astype(np.float32)
    model = ws.WarmStartModel(seed=3)
    r, t = torch.tensor(raw, device="cuda"), torch.tensor(target, device="cuda")
    model.fit_normalisation(r, t)
    losses = model.train(r, t, steps=400, batch=4096, lr=2e-3)
    assert np.mean(losses[-20:]) < 0.05 * np.mean(losses[:5])
    # forward matches the training loss on held-out rows
    y = model.forward(r[:4096]).cpu().numpy()
    tn = (target[:4096] - model.norm[-2]) / model.norm[-1]
    assert np.mean((y - tn) ** 2) < 0.1


def test_features_are_scaled_knn_distances(torch, ws):
    import geogram_gb300 as g
    x = np.random.default_rng(4).random((3000, 3))
    raw = ws.features(torch.tensor(x, device="cuda")).cpu().numpy()
    nn = g.NearestNeighborSearch(3)
    nn.set_points(x)
    _, d2 = nn.get_nearest_neighbors_by_index(17)
    assert np.allclose(raw[:, :3], x.astype(np.float32))
    ref = (np.sqrt(d2[:, 1:17]) * np.cbrt(3000)).astype(np.float32)
    assert np.allclose(raw[:, 3:], ref, rtol=1e-6, atol=1e-6)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(
    os.path.abspath(__file__))), "geogram_gb300", "data", "warmstart_mlp.npz")),
    reason="no trained model")
def test_trained_warm_start_reaches_the_tolerance(torch, ws):
    """The shipped network's start on a held-out mixture converges to the
    same mass tolerance as the zero start, within 3 Newton iterations of it.
    It does not beat the zero start (it is scaled toward zero when it empties
    a cell); both starts' Newton iterations, cell passes and times are
    printed."""
    import geogram_gb300 as g
    model = ws.WarmStartModel.load()
    rng = np.random.default_rng(123)
    x = torch.tensor(gaussian_mixture(30000, 9, rng.uniform(0.03, 0.09, 9), rng), device="cuda")
    w = torch.zeros(x.shape[0], dtype=torch.float64, device="cuda")
    plain = g.ot_solve_device(x, w, tol=1e-6)
    w1 = torch.empty_like(w)
    warm = model.solve(x, w1, tol=1e-6)
    print(f"\nplain: {plain['newton_iters']} Newton, {plain['cell_calls']} cell passes, "
          f"{plain['ms_total']:.0f} ms; learned start (scale {warm['start_scale']}): "
          f"{warm['newton_iters']} Newton, {warm['cell_calls']} cell passes, "
          f"{warm['ms_total']:.0f} ms")
    assert plain["converged"] == 1 and warm["converged"] == 1
    assert warm["mass_error_inf"] < 1e-6
    assert warm["newton_iters"] <= plain["newton_iters"] + 3
