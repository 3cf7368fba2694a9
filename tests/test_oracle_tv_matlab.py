"""The MATLAB TV restatements (oracle/tv_matlab.py) checked against each
other and against the scikit-image Chambolle restatement where the
reference files coincide.  No MATLAB output exists to pin them directly."""
import numpy as np
import pytest

from oracle import tv_matlab as tm
from oracle.tv_chambolle import _tv_chambolle_nd, tv_cham_itv2d_matlab


def stack(H, W, B, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W] / max(H, W)
    base = np.stack([np.sin(6 * xx + b) * np.cos(4 * yy - b) for b in range(B)], axis=2)
    return 0.5 + 0.3 * base + 0.05 * rng.standard_normal((H, W, B))


@pytest.mark.parametrize("tvm", sorted(tm.TVM))
def test_constant_frames_are_fixed_points(tvm):
    f = np.full((12, 17, 3), 0.4)
    f[..., 1] = 0.9
    assert np.allclose(tm.tv_by_name(f, tvm, 0.1), f, atol=1e-14)


@pytest.mark.parametrize("tvm", sorted(tm.TVM))
def test_output_is_finite_and_smoother(tvm):
    f = stack(20, 24, 4, seed=1)
    u = tm.tv_by_name(f, tvm, 0.1)
    assert u.shape == f.shape and np.all(np.isfinite(u))
    tv = lambda a: np.abs(np.diff(a, axis=0)).sum() + np.abs(np.diff(a, axis=1)).sum()  # noqa
    assert tv(u) < tv(f)


def test_single_frame_branches():
    """MATLAB treats an H x W x 1 stack as 2-D: ClipB then runs ClipA's
    update and ATV_cham the isotropic update; the coupled 3-D norms reduce
    to the per-frame ones."""
    f = stack(16, 21, 1, seed=2)
    assert np.array_equal(tm.tv_denoising_clip_lb(f, 0.1, 5), tm.tv_denoising(f, 0.1, 5))
    assert np.array_equal(tm.tvdenoise_cham_atv2d(f, 8.0, 5), tm.tvdenoise_cham_itv2d(f, 8.0, 5))
    assert np.allclose(tm.fgp_denoise_itv3d(f, 0.1, 3), tm.fgp_denoise_itv2d(f, 0.1, 3),
                       rtol=0, atol=1e-15)
    assert np.allclose(tm.tvdenoise_cham_itv3d(f, 8.0, 5), tm._cham(f, 8.0, 5, 1 / 4, "iso"),
                       rtol=0, atol=1e-15)
    # more than one frame takes the other branch
    g = stack(16, 21, 2, seed=2)
    assert not np.allclose(tm.tv_denoising_clip_lb(g, 0.1, 5), tm.tv_denoising(g, 0.1, 5))
    assert not np.allclose(tm.tvdenoise_cham_atv2d(g, 8.0, 5),
                           tm.tvdenoise_cham_itv2d(g, 8.0, 5))


@pytest.mark.parametrize("fn,param,it", [(tm.tv_denoising, 0.1, 5),
                                         (tm.tvdenoise_cham_itv2d, 10.0, 5),
                                         (tm.fgp_denoise_itv2d, 0.1, 3),
                                         (tm.fgp_denoise_atv2d, 0.1, 3),
                                         (tm.tv_denoising_clip_lb, 0.1, 5),
                                         (tm.tvdenoise_cham_atv2d, 10.0, 5)])
def test_per_frame_variants_are_frame_independent(fn, param, it):
    """Every variant but the ITV3D ones denoises each frame on its own (on a
    stack of more than one frame, i.e. in MATLAB's 3-D branch)."""
    f = stack(14, 19, 3, seed=3)
    u = fn(f, param, it)
    for b in range(3):
        g = np.concatenate([f[..., b:b + 1], f[..., b:b + 1]], axis=2)
        assert np.allclose(fn(g, param, it)[..., 0], u[..., b], rtol=0, atol=1e-15)


def test_itv3d_couples_frames():
    f = stack(14, 19, 3, seed=4)
    u = tm.tvdenoise_cham_itv3d(f, 8.0, 5)
    g = f.copy()
    g[..., 2] = 0.0
    assert not np.allclose(tm.tvdenoise_cham_itv3d(g, 8.0, 5)[..., 0], u[..., 0])
    # FGP projects only where the summed dual norm exceeds 1 (small lambda)
    v = tm.fgp_denoise_itv3d(f, 0.004, 3)
    assert not np.allclose(tm.fgp_denoise_itv3d(g, 0.004, 3)[..., 0], v[..., 0])


def test_itv2d_cham_matches_the_second_restatement():
    """Two independent restatements of tvdenoise_cham_ITV2D.m agree."""
    f = stack(23, 31, 1, seed=5)[..., 0]
    a = tm.tvdenoise_cham_itv2d(f, 7.0, 6)[..., 0]
    b = tv_cham_itv2d_matlab(f, 7.0, 6)
    assert np.allclose(a, b, rtol=0, atol=1e-14)


@pytest.mark.parametrize("iters", [1, 3, 5])
def test_itv3d_cham_is_the_skimage_recurrence_away_from_the_first_row_and_column(iters):
    """tvdenoise_cham_ITV3D on one frame (dt = 1/4, lambda = 1/w) is the
    scikit-image Chambolle recurrence without stop test: K MATLAB updates
    are K+1 scikit-image steps.  The files differ only in div p at the
    first row and column, which reaches `iters` pixels inward."""
    f = stack(30, 34, 1, seed=6)[..., 0]
    w = 0.15
    ml = tm.tvdenoise_cham_itv3d(f, 1.0 / w, iters)[..., 0]
    sk, steps, _ = _tv_chambolle_nd(f, w, 0.0, iters + 1)
    assert steps == iters + 1
    m = iters + 1
    assert np.allclose(ml[m:, m:], sk[m:, m:], rtol=0, atol=1e-12)
    assert not np.allclose(ml[:1], sk[:1], atol=1e-9)


def test_fgp_first_iterations():
    """FGP: one iteration returns Xobs; two return Xobs - lam L(P) with P
    the projected step from zero."""
    f = stack(10, 13, 2, seed=7)
    assert np.array_equal(tm.fgp_denoise_itv2d(f, 0.2, 1), f)
    lam = 0.2
    Q1, Q2 = tm._ltrans(f)
    P1, P2 = Q1 / (8 * lam), Q2 / (8 * lam)
    P1, P2 = P1 / np.maximum(np.abs(P1), 1), P2 / np.maximum(np.abs(P2), 1)
    ref = f - lam * tm._lforward(P1, P2)
    assert np.allclose(tm.fgp_denoise_atv2d(f, lam, 2), ref, rtol=0, atol=1e-15)


def test_clip_first_iteration_and_bound():
    f = stack(10, 13, 2, seed=8)
    assert np.array_equal(tm.tv_denoising(f, 0.1, 1), f)
    # the clipped duals bound the change of each pixel: |x0 - y0| <= 2 lam/2
    u = tm.tv_denoising(f, 0.1, 5)
    assert np.max(np.abs(u - f)) <= 0.1 + 1e-12


def test_gap_loop_with_matlab_tv_improves_psnr():
    rng = np.random.default_rng(9)
    H, W, B = 32, 36, 4
    x = stack(H, W, B, seed=9)
    mask = (rng.random((H, W, B)) < 0.5).astype(np.float64)
    y = np.sum(x * mask, axis=2)
    v0 = mask * y[:, :, None]
    for tvm in ("ATV_ClipA", "ITV3D_cham", "ITV2D_FGP"):
        v = tm.gap_tv_matlab(y, mask, tvm, 0.07, 12)
        assert np.mean((v - x) ** 2) < np.mean((v0 - x) ** 2)
