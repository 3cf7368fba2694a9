"""GPU joint TV + CNN loops (joint_pnp_sci_algo.py) against the reference's
own joint_admmdenoise_cacti run (golden fixtures, box-blur stand-in CNN)
and against the oracle's restatement for multi-block and flipped cases."""
import json

import numpy as np
import pytest
import torch
import torch.nn.functional as F

import sci_algorithms_gb300 as sci
from oracle import reference_port as port

pytestmark = pytest.mark.gpu

REL_L2 = 1e-4
PSNR_TOL = 1e-2


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def box_blur(x, nsig):
    """3 x 3 mean of every frame with replicated edges: the CNN plug-in the
    fixtures were made with (planar frames x H x W float32 CUDA in / out)."""
    p = F.pad(x[:, None], (1, 1, 1, 1), mode="replicate")
    return F.avg_pool2d(p, 3, stride=1)[:, 0]


def _args(g):
    return json.loads(str(g["args_json"]))


def _check(out, g):
    x_, _t, psnr_, ssim_, psnrall_ = out
    x_ = x_.cpu().numpy() if torch.is_tensor(x_) else x_
    assert x_.shape == g["x"].shape
    assert rel(x_, g["x"]) < REL_L2
    assert np.max(np.abs(np.array(psnr_) - g["psnr"])) < PSNR_TOL
    assert np.max(np.abs(np.array(ssim_) - g["ssim"])) < 1e-4
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < PSNR_TOL


@pytest.mark.parametrize("case", ["joint_gap", "joint_admm"])
def test_joint_native_matches_reference(golden, case):
    g = golden(case)
    A, At = sci.make_ops(g["mask"])
    out = sci.joint_admmdenoise_cacti(g["meas"], g["mask"], A, At, projmeth=case.split("_")[1],
                                      orig=g["orig"], denoiser=str(g["denoiser"]),
                                      model=box_blur, **_args(g))
    assert isinstance(out[0], np.ndarray) and out[0].dtype == np.float32
    _check(out, g)


@pytest.mark.parametrize("case", ["joint_gap", "joint_admm"])
def test_joint_plugin_operators_match_reference(golden, case):
    g = golden(case)
    mask = torch.from_numpy(g["mask"]).cuda()
    A = lambda x: sci.A_(x, mask)  # noqa: E731
    At = lambda y: sci.At_(y, mask)  # noqa: E731
    out = sci.joint_admmdenoise_cacti(torch.from_numpy(g["meas"]).cuda(), mask, A, At,
                                      projmeth=case.split("_")[1],
                                      orig=torch.from_numpy(g["orig"]).cuda(),
                                      denoiser=str(g["denoiser"]), model=box_blur, **_args(g))
    assert out[0].is_cuda
    _check(out, g)


@pytest.mark.parametrize("projmeth", ["gap", "admm"])
def test_joint_blocks_flip_and_start_point(projmeth):
    """Two coded frames, up-down mask direction, a given start point, a
    two-stage sigma list: against the oracle's restatement."""
    rng = np.random.default_rng(91)
    H, W, B = 20, 28, 6
    mask = (rng.random((H, W, B)) > 0.5).astype(np.float64)
    orig = rng.random((H, W, 2 * B))
    meas = np.stack([port.A_(orig[..., k * B:(k + 1) * B], mask) for k in range(2)], axis=-1)
    v0 = rng.random((H, W, 2 * B)) * 0.5
    args = dict(_lambda=1, tv_weight=0.1, tv_iter_max=5, sigma1=[None], sigma2=[0.05, 0.02],
                iter_max1=3, iter_max2=[2, 2])
    if projmeth == "admm":
        args["gamma"] = 0.03
    ref = port.joint_admmdenoise_cacti(meas, mask, lambda x: port.A_(x, mask),
                                       lambda y: port.At_(y, mask), port.cnn_stand_in,
                                       projmeth=projmeth, v0=v0, orig=orig, nframe=2,
                                       maskdirection="updown", denoiser="tv+ffdnet", **args)
    A, At = sci.make_ops(mask)
    out = sci.joint_admmdenoise_cacti(meas, mask, A, At, projmeth=projmeth, v0=v0, orig=orig,
                                      nframe=2, maskdirection="updown", denoiser="tv+ffdnet",
                                      model=box_blur, **args)
    assert rel(out[0], ref[0]) < REL_L2
    assert np.max(np.abs(np.array(out[2]) - np.array(ref[2]))) < PSNR_TOL
    assert np.max(np.abs(np.array(out[4]) - np.array(ref[4]))) < PSNR_TOL


def test_joint_rejects_bad_arguments(golden):
    g = golden("joint_gap")
    A, At = sci.make_ops(g["mask"])
    kw = dict(iter_max1=1, iter_max2=1, sigma1=[None], sigma2=[0.05])
    with pytest.raises(ValueError):
        sci.joint_admmdenoise_cacti(g["meas"], g["mask"], A, At, projmeth="gap",
                                    denoiser="tv+bm3d", model=box_blur, **kw)
    with pytest.raises(TypeError):
        sci.joint_admmdenoise_cacti(g["meas"], g["mask"], A, At, projmeth="gap",
                                    denoiser="tv+ffdnet", model=None, **kw)
    with pytest.raises(ValueError):
        sci.joint_admmdenoise_cacti(g["meas"], g["mask"], A, At, projmeth="gap",
                                    denoiser="tv+ffdnet", model=box_blur, tvm="ITV3D_FGP",
                                    **kw)
    with pytest.raises(ValueError):
        sci.joint_admmdenoise_cacti(g["meas"], g["mask"], A, At, projmeth="lsq",
                                    denoiser="tv+ffdnet", model=box_blur, **kw)
