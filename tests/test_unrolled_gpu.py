"""Differentiable unrolled GAP-TV: hand-written adjoints against FP64
central differences and plain-torch autograd of the same unrolled loop.

Tolerance: relative L2 <= 1e-4 between the float32 hand-written gradients
and float64 autograd (the bar for "matching gradients"); finite
differences in float64 with h = 1e-6 on 32 random coordinates.
"""
import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300.unrolled import torch_unrolled_loss, unrolled_loss

pytestmark = pytest.mark.gpu

GRAD_REL = 1e-4


def problem(N, B, H, W, K, seed=0):
    dev = torch.device("cuda")
    xs = [sci.datasets.video_scene(H, W, B, seed=seed + n) for n in range(N)]
    x_true = torch.from_numpy(np.stack([np.moveaxis(x, -1, 0) for x in xs])).float().to(dev)
    g = torch.Generator(device="cpu").manual_seed(seed)
    logits = torch.randn((B, H, W), generator=g).to(dev)
    lambdas = torch.full((K,), 0.1, device=dev)
    return logits, lambdas, x_true


def ours(logits, lambdas, x_true, K, T=5, w=0.1):
    lg = logits.clone().requires_grad_(True)
    lm = lambdas.clone().requires_grad_(True)
    loss = unrolled_loss(lg, lm, x_true, K=K, tv_iters=T, tv_weight=w)
    loss.backward()
    return loss.detach(), lg.grad.detach(), lm.grad.detach()


def torch_ref(logits, lambdas, x_true, K, T=5, w=0.1, dtype=torch.float64):
    lg = logits.detach().to(dtype).clone().requires_grad_(True)
    lm = lambdas.detach().to(dtype).clone().requires_grad_(True)
    loss = torch_unrolled_loss(lg, lm, x_true.to(dtype), K=K, tv_iters=T, tv_weight=w)
    loss.backward()
    return loss.detach(), lg.grad.detach(), lm.grad.detach()


def rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).norm() / b.norm())


@pytest.mark.parametrize("N,B,H,W,K,T", [(2, 8, 32, 40, 6, 5), (1, 4, 17, 23, 3, 3),
                                         (3, 8, 64, 64, 10, 5), (2, 6, 130, 260, 4, 2)])
def test_unrolled_matches_fp64_autograd(N, B, H, W, K, T):
    logits, lambdas, x_true = problem(N, B, H, W, K)
    l1, g1, m1 = ours(logits, lambdas, x_true, K, T)
    l2, g2, m2 = torch_ref(logits, lambdas, x_true, K, T)
    assert abs(float(l1) - float(l2)) <= 1e-5 * abs(float(l2))
    assert rel(g1, g2) < GRAD_REL, rel(g1, g2)
    assert rel(m1, m2) < GRAD_REL, rel(m1, m2)


@pytest.mark.parametrize("T", [5, 3])
def test_stored_tape_and_recompute_agree(monkeypatch, T):
    """The reverse pass on the tape the forward TV kept (SCI_UNROLLED_TAPE=1)
    against the default that recomputes it: the same adjoint of (almost)
    the same tape."""
    N, B, H, W, K = 2, 8, 48, 72, 5
    logits, lambdas, x_true = problem(N, B, H, W, K, seed=5)
    l2, g2, m2 = ours(logits, lambdas, x_true, K, T)
    monkeypatch.setenv("SCI_UNROLLED_TAPE", "1")
    l1, g1, m1 = ours(logits, lambdas, x_true, K, T)
    assert abs(float(l1) - float(l2)) <= 1e-6 * abs(float(l2))
    assert rel(g1, g2) < 1e-5
    assert rel(m1, m2) < 1e-5


def test_unrolled_central_differences():
    N, B, H, W, K = 2, 8, 24, 28, 20
    logits, lambdas, x_true = problem(N, B, H, W, K, seed=3)
    _, g, m = ours(logits, lambdas, x_true, K)
    lg64 = logits.double()
    lm64 = lambdas.double()
    xt64 = x_true.double()
    h = 1e-6
    rng = np.random.default_rng(0)
    idx = [tuple(int(rng.integers(0, s)) for s in logits.shape) for _ in range(32)]

    def L(a, b):
        return float(torch_unrolled_loss(a, b, xt64, K=K))
    gmax = float(g.abs().max())
    for i in idx:
        a, b = lg64.clone(), lg64.clone()
        a[i] += h
        b[i] -= h
        fd = (L(a, lm64) - L(b, lm64)) / (2 * h)
        assert abs(float(g[i]) - fd) <= 1e-3 * abs(fd) + 1e-4 * gmax, (i, float(g[i]), fd)
    for k in (0, 7, K - 1):
        a, b = lm64.clone(), lm64.clone()
        a[k] += h
        b[k] -= h
        fd = (L(lg64, a) - L(lg64, b)) / (2 * h)
        assert abs(float(m[k]) - fd) <= 1e-3 * abs(fd) + 1e-4 * float(m.abs().max()), (k, fd)


def test_unrolled_batch16_against_autograd():
    """The 16 x 256 x 256 x 8, K = 20 workload: hand-written vs FP32 and FP64
    autograd."""
    N, B, H, W, K = 16, 8, 256, 256, 20
    logits, lambdas, x_true = problem(N, B, H, W, K, seed=11)
    l1, g1, m1 = ours(logits, lambdas, x_true, K)
    l3, g3, m3 = torch_ref(logits, lambdas, x_true, K, dtype=torch.float32)
    l2, g2, m2 = torch_ref(logits, lambdas, x_true, K, dtype=torch.float64)
    print("unrolled 16x256x256x8: rel(logits grad) ours %.2e, torch-fp32 %.2e; "
          "rel(lambda grad) ours %.2e, torch-fp32 %.2e"
          % (rel(g1, g2), rel(g3, g2), rel(m1, m2), rel(m3, m2)))
    assert rel(g1, g2) < GRAD_REL
    assert rel(m1, m2) < GRAD_REL
    assert rel(g1, g3) < GRAD_REL
