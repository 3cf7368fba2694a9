"""Differentiable unrolled GAP-TV with hand-written adjoint kernels.

``UnrolledGapTV`` is a ``torch.autograd.Function`` over the C-ABI pair
``sci_unrolled_fwd`` / ``sci_unrolled_bwd``: a batch of scenes shares one
learnable coded mask (``Phi = sigmoid(logits)``) and per-iteration step
sizes ``lambdas``; the loss is the mean squared error of K unrolled
accelerated-GAP + TV iterations (the ``gap_denoise`` loop of
``PnP_SCI/python/pnp_sci_algo.py:636-650`` with a fixed number of Chambolle
steps and no stop test).  The forward keeps only the outer iterates; the
backward recomputes each TV call from its checkpoint.

``torch_unrolled_loss`` is the same loop in plain PyTorch ops (for the
autograd comparison and as a readable statement of the model).  Its norm
uses the same safe convention as the kernels: |g| has gradient 0 at g = 0.
"""
import ctypes

import torch

from . import _dev
from ._lib import call


class _Buffers:
    """Fixed device buffers of one workspace: inputs are copied in and
    outputs read out of them, so the cached CUDA graphs of the forward and
    reverse passes (keyed by pointers) are replayed on every call."""

    def __init__(self, N, B, H, W, K, dev):
        self.logits = torch.empty((B, H, W), dtype=torch.float32, device=dev)
        self.lambdas = torch.empty((K,), dtype=torch.float32, device=dev)
        self.x_true = torch.empty((N, B, H, W), dtype=torch.float32, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        self.glog = torch.empty((B, H, W), dtype=torch.float32, device=dev)
        self.glam = torch.zeros(K, dtype=torch.float64, device=dev)


_BUFFERS = {}


def _buffers(ws, N, B, H, W, K):
    key = (ws.data_ptr(), N, B, H, W, K)
    b = _BUFFERS.get(key)
    if b is None:
        b = _BUFFERS[key] = _Buffers(N, B, H, W, K, ws.device)
    return b


class UnrolledGapTV(torch.autograd.Function):
    @staticmethod
    def forward(ctx, logits, lambdas, x_true, K, tv_iters, tv_weight, ws=None):
        N, B, H, W = x_true.shape
        if ws is None:
            ws = unrolled_workspace(N, B, H, W, K, tv_iters, x_true.device)
        bf = _buffers(ws, N, B, H, W, K)
        bf.logits.copy_(logits.detach())
        bf.lambdas.copy_(lambdas.detach())
        bf.x_true.copy_(x_true.detach())
        call("sci_unrolled_fwd", bf.logits.data_ptr(), bf.lambdas.data_ptr(),
             bf.x_true.data_ptr(), N, B, H, W, K, tv_iters, float(tv_weight), bf.loss.data_ptr(),
             None, ws.data_ptr(), ws.numel(), _dev.stream_handle())
        ctx.ws, ctx.bf = ws, bf
        ctx.cfg = (N, B, H, W, K, tv_iters, float(tv_weight))
        return (bf.loss / x_true.numel()).to(torch.float32).reshape(())

    @staticmethod
    def backward(ctx, grad):
        N, B, H, W, K, T, w = ctx.cfg
        bf, ws = ctx.bf, ctx.ws
        call("sci_unrolled_bwd", bf.logits.data_ptr(), bf.lambdas.data_ptr(),
             bf.x_true.data_ptr(), N, B, H, W, K, T, w, float(grad.item()), bf.glog.data_ptr(),
             bf.glam.data_ptr(), ws.data_ptr(), ws.numel(), _dev.stream_handle())
        return bf.glog.clone(), bf.glam.to(torch.float32), None, None, None, None, None


def unrolled_loss(logits, lambdas, x_true, K=20, tv_iters=5, tv_weight=0.1, ws=None):
    """MSE of the K-iteration unrolled GAP-TV (hand-written forward/backward)."""
    return UnrolledGapTV.apply(logits, lambdas, x_true, K, tv_iters, tv_weight, ws)


def unrolled_workspace(N, B, H, W, K=20, tv_iters=5, dev=None):
    n = ctypes.c_size_t()
    call("sci_unrolled_workspace_bytes", N, B, H, W, K, tv_iters, ctypes.byref(n))
    return _dev.workspace(n.value, dev)


# ------------------------------------------------------------ plain torch
def _safe_norm(a, b):
    s = a * a + b * b
    pos = s > 0
    return torch.where(pos, torch.sqrt(torch.where(pos, s, torch.ones_like(s))),
                       torch.zeros_like(s))


def _grad(u):
    gr = torch.zeros_like(u)
    gc = torch.zeros_like(u)
    gr[..., :-1, :] = u[..., 1:, :] - u[..., :-1, :]
    gc[..., :, :-1] = u[..., :, 1:] - u[..., :, :-1]
    return gr, gc


def _div(pr, pc):
    d = pr + pc
    d = d - torch.nn.functional.pad(pr[..., :-1, :], (0, 0, 1, 0))
    d = d - torch.nn.functional.pad(pc[..., :, :-1], (1, 0, 0, 0))
    return d


def torch_tv(f, weight, steps):
    """Chambolle TV with a fixed number of steps (no stop test), plain ops."""
    tau = 0.25
    pr = torch.zeros_like(f)
    pc = torch.zeros_like(f)
    u = f
    for _ in range(steps - 1):
        gr, gc = _grad(u)
        n = _safe_norm(gr, gc)
        den = 1.0 + (tau / weight) * n
        pr = (pr - tau * gr) / den
        pc = (pc - tau * gc) / den
        u = f - _div(pr, pc)
    return u


def torch_unrolled_loss(logits, lambdas, x_true, K=20, tv_iters=5, tv_weight=0.1):
    """The unrolled GAP-TV loss in plain PyTorch (any dtype / device)."""
    phi = torch.sigmoid(logits)                      # B, H, W
    ps = phi.sum(0)
    y = (x_true * phi).sum(1)                        # N, H, W
    x = phi * (y / ps).unsqueeze(1)
    y1 = torch.zeros_like(y)
    for k in range(K):
        yb = (x * phi).sum(1)
        y1 = y1 + (y - yb)
        v = x + lambdas[k] * (phi * ((y1 - yb) / ps).unsqueeze(1))
        x = torch_tv(v, tv_weight, tv_iters)
    return ((x - x_true) ** 2).mean()
