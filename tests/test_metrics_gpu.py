"""GPU per-frame PSNR / SSIM (sci_frame_metrics) against the oracle's
restatement of scikit-image 0.16's compare_psnr / compare_ssim."""
import numpy as np
import pytest
import torch

from oracle import reference_port as port
from sci_algorithms_gb300.metrics import frame_psnr_ssim

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("B,H,W", [(1, 7, 7), (3, 9, 13), (2, 64, 80), (4, 130, 257)])
def test_frame_metrics_match_scikit_image_restatement(B, H, W):
    rng = np.random.default_rng(B * 100 + H)
    a = rng.random((B, H, W)).astype(np.float32)
    b = np.clip(a + 0.05 * rng.standard_normal(a.shape), 0, 1).astype(np.float32)
    psnr, ssim = frame_psnr_ssim(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    for f in range(B):
        ra = a[f].astype(np.float64)
        rb = b[f].astype(np.float64)
        assert abs(psnr[f] - port.compare_psnr(ra, rb, data_range=1.)) < 1e-9
        assert abs(ssim[f] - port.compare_ssim(ra, rb, data_range=1.)) < 1e-6


def test_frame_metrics_smooth_and_identical_frames():
    """Smooth frames (small local variance next to a large mean: where
    E[x^2] - E[x]^2 cancels) and identical frames (SSIM 1, PSNR inf)."""
    y, x = np.mgrid[0:96, 0:128] / 128.0
    a = (0.6 + 0.01 * np.sin(7 * x) * np.cos(5 * y))[None].astype(np.float32)
    b = (a + 1e-3 * np.cos(3 * x + y)[None]).astype(np.float32)
    psnr, ssim = frame_psnr_ssim(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    assert abs(ssim[0] - port.compare_ssim(a[0].astype(np.float64), b[0].astype(np.float64),
                                           data_range=1.)) < 1e-6
    p2, s2 = frame_psnr_ssim(torch.from_numpy(a).cuda(), torch.from_numpy(a).cuda())
    assert p2[0] == float("inf") and abs(s2[0] - 1.0) < 1e-12
    with pytest.raises(ValueError):
        frame_psnr_ssim(torch.zeros(1, 6, 9).cuda(), torch.zeros(1, 6, 9).cuda())
