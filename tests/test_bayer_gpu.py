"""GPU Bayer GAP-TV / ADMM-TV (pnp_sci_algo.py:20-476) against the
reference's own gap_denoise_bayer output (golden fixtures) and the ADMM
restatement (the reference's ADMM variant cannot run: it reads its
multiplier before assigning it, :400)."""
import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from oracle import reference_port as port

pytestmark = pytest.mark.gpu

REL_L2 = 1e-4
PSNR_TOL = 1e-2


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("case", ["bayer_gap", "bayer_gap_acc"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_gap_bayer_matches_reference(golden, case, use_graph):
    g = golden(case)
    x, psnr_, ssim_, psnr_all = sci.gap_denoise_bayer(
        g["meas"], g["mask"], _lambda=1, accelerate=bool(g["accelerate"]), iter_max=8,
        tv_weight=0.1, tv_iter_max=5, X_orig=g["orig"], use_graph=use_graph)
    assert x.shape == g["x"].shape and x.dtype == np.float32
    assert rel(x, g["x"]) < REL_L2
    assert np.max(np.abs(np.array(psnr_) - g["psnr"])) < PSNR_TOL
    assert np.max(np.abs(np.array(ssim_) - g["ssim"])) < 1e-4
    assert np.max(np.abs(np.array(psnr_all) - g["psnrall"])) < PSNR_TOL


def test_admm_bayer_matches_restatement(golden):
    g = golden("bayer_gap")
    ref, ref_psnr = port.admm_denoise_bayer(g["meas"], g["mask"], gamma=0.02, iter_max=6,
                                            tv_weight=0.1, X_orig=g["orig"])
    x, psnr_all = sci.admm_denoise_bayer(g["meas"], g["mask"], gamma=0.02, iter_max=6,
                                         tv_weight=0.1, X_orig=g["orig"])
    assert rel(x, ref) < REL_L2
    assert np.max(np.abs(np.array(psnr_all) - np.array(ref_psnr))) < PSNR_TOL


def test_bayer_torch_inputs_x0_and_odd_sizes(golden):
    g = golden("bayer_gap_acc")
    y = torch.from_numpy(g["meas"]).cuda()
    m = torch.from_numpy(g["mask"]).cuda()
    x, _, _, _ = sci.gap_denoise_bayer(y, m, iter_max=8, tv_weight=0.1)
    assert x.is_cuda and rel(x.cpu().numpy(), g["x"]) < REL_L2
    # a given start point is split like the measurement (:136-137)
    x0 = np.asarray(g["x"])
    ref, _, _, _ = port.gap_denoise_bayer(g["meas"], g["mask"], iter_max=3, tv_weight=0.1,
                                          x0_bayer=x0)
    x2, _, _, _ = sci.gap_denoise_bayer(g["meas"], g["mask"], iter_max=3, tv_weight=0.1,
                                        x0_bayer=x0)
    assert rel(x2, ref) < REL_L2
    with pytest.raises(ValueError):
        sci.gap_denoise_bayer(g["meas"][:-1], g["mask"][:-1], iter_max=1)
