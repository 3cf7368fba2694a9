"""Per-frame image-quality metrics the solvers report, computed on the GPU.

``frame_psnr`` / ``frame_ssim`` follow scikit-image 0.16's
``measure.compare_psnr`` and ``measure.compare_ssim`` with the options the
reference passes (``PnP_SCI/python/pnp_sci_algo.py:702-705``, ``:860-863``:
``data_range=1``, defaults otherwise): PSNR = 10 log10(R^2 / MSE); SSIM of
Wang et al. (2004) with a 7 x 7 uniform window, sample covariance
N/(N-1), K1 = 0.01, K2 = 0.03, averaged over the image cropped by 3 pixels
(whose windows never reach the border extension).  Both come from one
pass of ``sci_frame_metrics`` (float32 centred window moments, float64
sums).
"""
import math

import torch

from . import _dev
from ._lib import call


def frame_psnr_ssim(orig_planar, x_planar, data_range=1.0):
    """(PSNR list, SSIM list) per frame of planar (B, H, W) stacks."""
    o = orig_planar.to(torch.float32).contiguous()
    x = x_planar.to(device=o.device, dtype=torch.float32).contiguous()
    if o.shape != x.shape or o.dim() != 3:
        raise ValueError("frame stacks of equal (B, H, W) shape expected")
    B, H, W = o.shape
    if H < 7 or W < 7:
        raise ValueError("SSIM needs frames of at least 7 x 7 (win_size 7)")
    out = torch.empty((2, B), dtype=torch.float64, device=o.device)
    call("sci_frame_metrics", o.data_ptr(), x.data_ptr(), B, H, W, float(data_range),
         out[0].data_ptr(), out[1].data_ptr(), _dev.stream_handle())
    se, ss = out.cpu().tolist()
    psnr = [10 * math.log10(data_range ** 2 / (e / (H * W))) if e > 0 else float("inf")
            for e in se]
    ssim = [v / ((H - 6) * (W - 6)) for v in ss]
    return psnr, ssim


def frame_psnr(orig_planar, x_planar, data_range=1.0):
    """compare_psnr per frame of planar (B, H, W) stacks -> list of floats."""
    return frame_psnr_ssim(orig_planar, x_planar, data_range)[0]


def frame_ssim(orig_planar, x_planar, data_range=1.0):
    """compare_ssim per frame of planar (B, H, W) stacks -> list of floats."""
    return frame_psnr_ssim(orig_planar, x_planar, data_range)[1]
