"""GPU MATLAB-twin TV denoisers (sci_tv_matlab) against the oracle
restatements of PnP_SCI/matlab/algorithms/tvdenoisers/*.m, alone and inside
the GAP / ADMM loops (native graph path and plug-in path)."""
import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev
from sci_algorithms_gb300._lib import SciError
from oracle import tv_matlab as tm

pytestmark = pytest.mark.gpu

# float32 kernels vs float64 oracle on images with values in [0, 1]
ATOL = 2e-5
REL_L2 = 1e-4


def frames(H, W, B, seed):
    rng = np.random.default_rng(seed)
    base = sci.datasets.video_scene(H, W, B, seed=seed) if min(H, W) >= 8 else \
        rng.random((H, W, B))
    return np.clip(base + 0.05 * rng.standard_normal((H, W, B)), 0, 1)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("tvm", sorted(sci.TVM))
@pytest.mark.parametrize("H,W,B", [(2, 2, 1), (5, 3, 2), (37, 61, 3), (64, 128, 1),
                                   (130, 260, 4), (256, 256, 8)])
def test_denoiser_matches_oracle(tvm, H, W, B):
    f = frames(H, W, B, seed=H * 7 + W + B)
    for w in (0.07, 0.3):
        ref = tm.tv_by_name(f, tvm, w)
        out = sci.denoise_tv_matlab(f, tvm, w)
        assert out.shape == f.shape and out.dtype == f.dtype
        assert np.max(np.abs(out - ref)) < ATOL, (tvm, w)


@pytest.mark.parametrize("tvm,lam", [("ITV3D_FGP", 0.004), ("ITV2D_FGP", 0.004),
                                     ("ATV_FGP", 0.004), ("ITV3D_cham", 2.0)])
@pytest.mark.parametrize("iters", [1, 2, 4, 6, 11])
def test_projection_active_and_iteration_counts(tvm, lam, iters):
    """Small FGP lambdas make the dual projection bind (and couple the
    frames for ITV3D); other iteration counts than gapdenoise's (ITV3D
    Chambolle runs passes of up to 5 updates: 6 and 11 carry the dual field
    through the workspace between passes)."""
    f = frames(48, 40, 3, seed=iters)
    kind = sci.TVM[tvm][0]
    fn = tm._FN[tm.TVM[tvm][0]]
    ref = fn(f, lam, iters)
    u = sci.tv_matlab_frames(_dev.planar(f), kind, lam, iters)
    torch.cuda.synchronize()
    # FGP with a small lambda amplifies float32 rounding by 1/(8 lambda)
    assert np.max(np.abs(_dev.unplanar(u, f) - ref)) < (2e-4 if "FGP" in tvm else ATOL)


@pytest.mark.parametrize("B", [5, 7, 22, 31, 32])
@pytest.mark.parametrize("H,W", [(33, 70), (17, 9)])
def test_itv3d_frame_counts(B, H, W):
    """ITV3D Chambolle with frame counts that leave frame lanes idle (the
    norm over frames is reduced across lanes) and strips narrower than a
    warp's 8 columns."""
    f = frames(H, W, B, seed=B + H)
    ref = tm.tv_by_name(f, "ITV3D_cham", 0.1)
    out = sci.denoise_tv_matlab(f, "ITV3D_cham", 0.1)
    assert np.max(np.abs(out - ref)) < ATOL


@pytest.mark.parametrize("H,W,B,iters", [(300, 260, 24, 5), (129, 517, 32, 5), (64, 1000, 16, 2),
                                         (97, 45, 12, 7)])
def test_itv3d_row_chunks_and_strips(H, W, B, iters):
    """ITV3D Chambolle at sizes with many row chunks (each recomputes the
    2 S + 1 rows around its edges) and column strips (each owns 32 - 2 S - 1
    columns of its 32 lanes)."""
    f = frames(H, W, B, seed=H + W + B)
    ref = tm.tvdenoise_cham_itv3d(f, 10.0, iters)
    u = sci.tv_matlab_frames(_dev.planar(f), sci.TVM["ITV3D_cham"][0], 10.0, iters)
    torch.cuda.synchronize()
    assert np.max(np.abs(_dev.unplanar(u, f) - ref)) < ATOL


def test_one_frame_takes_matlabs_2d_branch():
    f = frames(40, 52, 1, seed=5)
    a = sci.denoise_tv_matlab(f, "ATV_ClipB", 0.1)
    b = sci.denoise_tv_matlab(f, "ATV_ClipA", 0.1)
    assert np.array_equal(a, b)
    c = sci.denoise_tv_matlab(f, "ATV_cham", 0.1)
    d = sci.denoise_tv_matlab(f, "ITV2D_cham", 0.1)
    assert np.array_equal(c, d)


def test_bad_arguments_raise():
    f = _dev.planar(frames(8, 8, 2, seed=1))
    with pytest.raises(SciError):
        sci.tv_matlab_frames(f, 9, 0.1, 5)
    with pytest.raises(SciError):
        sci.tv_matlab_frames(f, 1, -0.1, 5)
    with pytest.raises(SciError):
        sci.tv_matlab_frames(_dev.planar(frames(1, 8, 2, seed=1)), 1, 0.1, 5)
    with pytest.raises(ValueError):
        sci.denoise_tv_matlab(frames(8, 8, 2, seed=1), "ATV_ClipC", 0.1)


def admm_tv_matlab(y, mask, tvm, w, iters, gamma=0.01, lam=1.0):
    """float64 ADMM loop of pnp_sci_algo.py:800-862 with a MATLAB-twin TV."""
    phisum = mask.sum(axis=2)
    phisum[phisum == 0] = 1
    theta = mask * y[:, :, None]
    b = np.zeros_like(theta)
    x = theta
    for _ in range(iters):
        t = theta + b
        yb = np.sum(t * mask, axis=2)
        x = t + lam * (mask * ((y - yb) / (phisum + gamma))[:, :, None])
        v = x - b
        theta = tm.tv_by_name(v, tvm, w)
        b = b - (x - theta)
    return x


@pytest.mark.parametrize("tvm", sorted(sci.TVM))
def test_gap_loop_native_and_plugin(tvm):
    orig, mask, meas = sci.datasets.video_config(48, 64, 8)
    ref = tm.gap_tv_matlab(meas, mask, tvm, 0.07, 10)
    A, At = sci.make_ops(mask)
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    for use_graph in (True, False):
        x, _, _, _ = sci.gap_denoise(meas, msum, A, At, _lambda=1, accelerate=True, iter_max=10,
                                     tv_weight=0.07, tvm=tvm, use_graph=use_graph,
                                     show_iqa=False)
        assert rel(x, ref) < REL_L2, (tvm, use_graph)
    Ap = lambda v: sci.A_(v, mask)  # noqa: E731  foreign callables: plug-in loop
    Atp = lambda r: sci.At_(r, mask)  # noqa: E731
    x, _, _, _ = sci.gap_denoise(meas, msum, Ap, Atp, _lambda=1, accelerate=True, iter_max=10,
                                 tv_weight=0.07, tvm=tvm, show_iqa=False)
    assert rel(x, ref) < REL_L2, tvm


@pytest.mark.parametrize("tvm", ["ATV_ClipA", "ITV3D_cham", "ITV2D_FGP"])
def test_admm_loop_native(tvm):
    orig, mask, meas = sci.datasets.video_config(40, 56, 8)
    ref = admm_tv_matlab(meas, mask, tvm, 0.1, 8)
    A, At = sci.make_ops(mask)
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    x, _, _, _ = sci.admm_denoise(meas, msum, A, At, _lambda=1, gamma=0.01, iter_max=8,
                                  tv_weight=0.1, tvm=tvm, show_iqa=False)
    assert rel(x, ref) < REL_L2


def test_cacti_driver_with_matlab_tv_and_steps():
    orig, mask, meas = sci.datasets.video_config(32, 48, 8)
    A, At = sci.make_ops(mask)
    x_, t_, psnr_, ssim_, psnrall_ = sci.admmdenoise_cacti(
        meas[..., None], mask, A, At, projmeth="gap", orig=orig, _lambda=1, accelerate=True,
        iter_max=6, tv_weight=0.07, tvm="ITV2D_cham")
    assert x_.shape == (32, 48, 8) and len(psnrall_[0]) == 6
    op = sci.MaskOperator(mask)
    s = sci.Solver(op, "gap", 4, 1.0, 0.07, tvm="ITV2D_FGP")
    s.run(_dev.plane(meas), tv_steps=True)
    assert torch.all(s.tv_steps == 2)


@pytest.mark.parametrize("tvm,lam", [("ATV_ClipA", 0.1), ("ATV_ClipB", 0.05),
                                     ("ATV_cham", 12.0), ("ITV2D_cham", 12.0)])
@pytest.mark.parametrize("iters", [1, 2, 5, 6, 9])
@pytest.mark.parametrize("H,W,B", [(70, 130, 3), (300, 517, 2)])
def test_pipeline_kinds_any_iteration_count(tvm, lam, iters, H, W, B):
    """The clip and per-frame Chambolle files on the temporally blocked
    pipeline: one pass (<= 4 dual updates), several passes carrying p
    through the workspace, and the copy for no update; odd widths use the
    scalar edge path."""
    f = frames(H, W, B, seed=iters + W)
    kind = sci.TVM[tvm][0]
    ref = tm._FN[tm.TVM[tvm][0]](f, lam, iters)
    u = sci.tv_matlab_frames(_dev.planar(f), kind, lam, iters)
    torch.cuda.synchronize()
    assert np.max(np.abs(_dev.unplanar(u, f) - ref)) < ATOL, (tvm, iters)
