"""GPU parity of the mask operators and projections against the oracle."""
import ctypes

import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev
from sci_algorithms_gb300._lib import call
from oracle import reference_port as port

pytestmark = pytest.mark.gpu

# float32 arithmetic against float64 references
RTOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_A_At_golden(golden):
    g = golden("ops")
    assert rel(sci.A_(g["x"], g["phi"]), g["A"]) < RTOL
    assert rel(sci.At_(g["y"], g["phi"]), g["At"]) < RTOL
    assert abs(sci.psnr(g["x"], g["x"] + 0.01 * g["y"][..., None]) - g["psnr"]) < 1e-4
    assert sci.psnr(g["x"], g["x"]) == 100


@pytest.mark.parametrize("shape", [(1, 1, 1), (7, 13, 3), (64, 64, 8), (33, 250, 24),
                                   (256, 256, 32), (17, 20, 40)])
def test_A_At_shapes_and_adjoint(shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    phi = rng.random(shape)
    y = rng.standard_normal(shape[:2])
    assert rel(sci.A_(x, phi), port.A_(x, phi)) < RTOL
    assert rel(sci.At_(y, phi), port.At_(y, phi)) < RTOL
    # <A x, y> = <x, At y>
    lhs = float(np.sum(sci.A_(x, phi).astype(np.float64) * y))
    rhs = float(np.sum(x * sci.At_(y, phi).astype(np.float64)))
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + np.abs(x).sum())


def test_torch_views_are_used_without_copy():
    dev = _dev.device()
    xp = torch.randn(8, 32, 48, device=dev)
    view = xp.permute(1, 2, 0)
    assert _dev.planar(view).data_ptr() == xp.data_ptr()
    phi = (torch.rand(8, 32, 48, device=dev) < 0.5).float()
    y = sci.A_(view, phi.permute(1, 2, 0))
    assert y.is_cuda and tuple(y.shape) == (32, 48)
    ref = (xp.double() * phi.double()).sum(0)
    assert torch.allclose(y.double(), ref, rtol=1e-5, atol=1e-5)


def test_phisum_guard_and_mask_packing():
    rng = np.random.default_rng(3)
    mask = (rng.random((40, 44, 8)) < 0.5).astype(np.float64)
    mask[0, 0, :] = 0
    op = sci.MaskOperator(mask)
    ref = mask.sum(axis=2)
    ref[ref == 0] = 1
    assert np.array_equal(op.phisum.cpu().numpy(), ref.astype(np.float32))
    assert op.bits is not None
    bits = op.bits.cpu().numpy().view(np.uint32)
    for b in range(8):
        assert np.array_equal((bits >> b) & 1, mask[..., b].astype(np.uint32))
    frac = mask.copy()
    frac[3, 3, 2] = 0.5
    assert sci.MaskOperator(frac).bits is None
    assert sci.MaskOperator(np.ones((8, 8, 33))).bits is None  # B > 32


@pytest.mark.parametrize("accelerate", [True, False])
@pytest.mark.parametrize("packed", [True, False])
@pytest.mark.parametrize("W", [64, 61])
def test_proj_gap_matches_reference_step(accelerate, packed, W):
    rng = np.random.default_rng(11)
    H, B = 37, 8
    mask = (rng.random((H, W, B)) < 0.5).astype(np.float64)
    x = rng.random((H, W, B))
    y = rng.random((H, W)) * 4
    y1 = rng.random((H, W))
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    lam = 0.9
    # reference step (pnp_sci_algo.py:640-645)
    yb = port.A_(x, mask)
    if accelerate:
        y1r = y1 + (y - yb)
        xr = x + lam * port.At_((y1r - yb) / msum, mask)
    else:
        xr = x + lam * port.At_((y - yb) / msum, mask)
    op = sci.MaskOperator(mask, pack=packed)
    assert (op.bits is not None) == packed
    # keep every device buffer referenced until the kernel has run
    xd, y1d, yd, psd = _dev.planar(x), _dev.plane(y1), _dev.plane(y), _dev.plane(msum)
    out = torch.empty_like(xd)
    call("sci_proj_gap", xd.data_ptr(), op.phi.data_ptr(), _dev.ptr(op.bits), yd.data_ptr(),
         y1d.data_ptr(), psd.data_ptr(), out.data_ptr(), lam, int(accelerate), B, H, W,
         _dev.stream_handle())
    assert rel(_dev.unplanar(out, x), xr) < RTOL
    if accelerate:
        assert rel(y1d.cpu().numpy(), y1r) < RTOL


def test_proj_gap_unit_mask_one_frame_gives_y():
    """Known answer: Phi = 1, B = 1, lambda = 1 -- one GAP projection maps
    any x to y (pnp_sci_algo.py:645 with A x = x, Phi_sum = 1)."""
    rng = np.random.default_rng(12)
    H, W = 33, 64
    mask = np.ones((H, W, 1))
    x = rng.random((H, W, 1))
    y = rng.random((H, W))
    op = sci.MaskOperator(mask)
    xd, yd = _dev.planar(x), _dev.plane(y)
    y1d = torch.zeros_like(yd)
    psd = _dev.plane(np.ones((H, W)))
    out = torch.empty_like(xd)
    call("sci_proj_gap", xd.data_ptr(), op.phi.data_ptr(), _dev.ptr(op.bits), yd.data_ptr(),
         y1d.data_ptr(), psd.data_ptr(), out.data_ptr(), 1.0, 0, 1, H, W, _dev.stream_handle())
    np.testing.assert_allclose(out[0].cpu().numpy(), y.astype(np.float32), rtol=0, atol=1e-6)


def device_status():
    v = ctypes.c_uint(0)
    call("sci_device_status", ctypes.byref(v), 1)
    return v.value


@pytest.mark.parametrize("tile", ["256", "128", "512"])
@pytest.mark.parametrize("B,H,W", [(1, 16, 16), (8, 37, 64), (24, 130, 260), (32, 64, 96),
                                   (24, 512, 512), (8, 37, 61)])
def test_proj_gap_bulk_copy_kernel_is_bitwise_equal(monkeypatch, B, H, W, tile):
    """The bulk-copy (TMA) staged projection against the register/shared
    memory kernel: identical x_out and y1, including partial last tiles,
    32 frames, grids with several tiles per block, and W % 4 != 0 (which
    the bulk-copy path declines)."""
    rng = np.random.default_rng(B * 1000 + W)
    mask = (rng.random((H, W, B)) < 0.5).astype(np.float64)
    op = sci.MaskOperator(mask)
    assert op.bits is not None
    x = _dev.planar(rng.random((H, W, B)))
    y = _dev.plane(rng.random((H, W)) * 4)
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    ps = _dev.plane(msum)
    monkeypatch.setenv("SCI_PROJ_TP", tile)
    outs = []
    for tma in ("1", "0"):
        monkeypatch.setenv("SCI_PROJ_TMA", tma)
        for acc in (1, 0):
            y1 = _dev.plane(np.full((H, W), 0.25))
            out = torch.empty_like(x)
            call("sci_proj_gap", x.data_ptr(), None, op.bits.data_ptr(), y.data_ptr(),
                 y1.data_ptr(), ps.data_ptr(), out.data_ptr(), 0.7, acc, B, H, W,
                 _dev.stream_handle())
            torch.cuda.synchronize()
            outs.append((out.clone(), y1.clone()))
    for (a, ya), (b, yb) in zip(outs[:2], outs[2:]):
        assert torch.equal(a, b)
        assert torch.equal(ya, yb)
    assert device_status() == 0


@pytest.mark.parametrize("tile", ["128", "64", "256"])
@pytest.mark.parametrize("B,H,W", [(1, 16, 16), (8, 37, 64), (24, 130, 260), (32, 64, 96),
                                   (24, 512, 512)])
def test_proj_admm_bulk_copy_kernel_is_bitwise_equal(monkeypatch, B, H, W, tile):
    """The bulk-copy staged ADMM projection against the shared-memory
    kernel: identical v and x (with and without x), partial last tiles."""
    rng = np.random.default_rng(B * 7 + W)
    mask = (rng.random((H, W, B)) < 0.5).astype(np.float64)
    op = sci.MaskOperator(mask)
    th = _dev.planar(rng.random((H, W, B)))
    bb = _dev.planar(0.1 * rng.standard_normal((H, W, B)))
    y = _dev.plane(rng.random((H, W)) * 4)
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    ps = _dev.plane(msum)
    monkeypatch.setenv("SCI_PROJ_TP", tile)
    outs = []
    for tma in ("1", "0"):
        monkeypatch.setenv("SCI_PROJ_TMA", tma)
        for want_x in (True, False):
            v = torch.empty_like(th)
            x = torch.empty_like(th) if want_x else None
            call("sci_proj_admm", th.data_ptr(), bb.data_ptr(), None, op.bits.data_ptr(),
                 y.data_ptr(), ps.data_ptr(), v.data_ptr(), _dev.ptr(x), 0.9, 0.01, B, H, W,
                 _dev.stream_handle())
            torch.cuda.synchronize()
            outs.append((v.clone(), None if x is None else x.clone()))
    for (va, xa), (vb, xb) in zip(outs[:2], outs[2:]):
        assert torch.equal(va, vb)
        assert (xa is None and xb is None) or torch.equal(xa, xb)
    assert device_status() == 0


def test_bounded_wait_reports_and_the_context_survives():
    """A bulk-copy wait that runs out (a barrier nothing completes) sets the
    status bit instead of hanging; the next kernels run normally."""
    assert device_status() == 0
    call("sci_selftest_bounded_wait", 1000, _dev.stream_handle())
    torch.cuda.synchronize()
    assert device_status() == 1  # read and cleared
    assert device_status() == 0
    # the context is intact: a projection still matches the oracle step
    test_proj_gap_matches_reference_step(True, True, 64)


@pytest.mark.parametrize("packed", [True, False])
def test_proj_admm_matches_reference_step(packed):
    rng = np.random.default_rng(12)
    H, W, B = 29, 40, 6
    mask = (rng.random((H, W, B)) < 0.5).astype(np.float64)
    th = rng.random((H, W, B))
    b = rng.standard_normal((H, W, B)) * 0.1
    y = rng.random((H, W)) * 3
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    lam, gamma = 1.0, 0.05
    yb = port.A_(th + b, mask)
    xr = (th + b) + lam * port.At_((y - yb) / (msum + gamma), mask)
    op = sci.MaskOperator(mask, pack=packed)
    v = torch.empty((B, H, W), device=op.dev)
    xo = torch.empty_like(v)
    thd, bd, yd, psd = _dev.planar(th), _dev.planar(b), _dev.plane(y), _dev.plane(msum)
    call("sci_proj_admm", thd.data_ptr(), bd.data_ptr(), op.phi.data_ptr(), _dev.ptr(op.bits),
         yd.data_ptr(), psd.data_ptr(), v.data_ptr(), xo.data_ptr(), lam, gamma, B, H, W,
         _dev.stream_handle())
    assert rel(_dev.unplanar(xo, th), xr) < RTOL
    assert rel(_dev.unplanar(v, th), xr - b) < RTOL
