"""Per-frame image-quality metrics the solvers report, computed on the GPU.

``compare_psnr`` / ``compare_ssim`` follow scikit-image 0.16's
``measure.compare_psnr`` and ``measure.compare_ssim`` with the options the
reference passes (``PnP_SCI/python/pnp_sci_algo.py:702-705``, ``:860-863``:
``data_range=1``, defaults otherwise): PSNR = 10 log10(R^2 / MSE); SSIM of
Wang et al. (2004) with a 7 x 7 uniform window, 'reflect' borders, sample
covariance N/(N-1), K1 = 0.01, K2 = 0.03, averaged over the image cropped by
3 pixels.  They are diagnostics evaluated once per solve, in float64.
"""
import math

import torch
import torch.nn.functional as F


def _reflect_index(n, pad, dev):
    # half-sample symmetric extension: (c b a | a b c ... x y z | z y x)
    i = torch.arange(-pad, n + pad, device=dev)
    i = torch.where(i < 0, -i - 1, i)
    i = torch.where(i >= n, 2 * n - i - 1, i)
    return i


def _uniform(x, win):
    """scipy.ndimage.uniform_filter(x, win, mode='reflect') on (F, H, W)."""
    pad = win // 2
    F_, H, W = x.shape
    iy = _reflect_index(H, pad, x.device)
    ix = _reflect_index(W, pad, x.device)
    xp = x.index_select(1, iy).index_select(2, ix)
    return F.avg_pool2d(xp.unsqueeze(1), win, stride=1).squeeze(1)


def frame_psnr(orig_planar, x_planar, data_range=1.0):
    """compare_psnr per frame of planar (B, H, W) stacks -> list of floats."""
    d = orig_planar.double() - x_planar.double()
    mse = (d * d).mean(dim=(1, 2)).tolist()
    return [10 * math.log10(data_range ** 2 / m) if m > 0 else float("inf") for m in mse]


def frame_ssim(orig_planar, x_planar, data_range=1.0, win=7):
    """compare_ssim per frame of planar (B, H, W) stacks -> list of floats."""
    X = orig_planar.double()
    Y = x_planar.double()
    npix = win * win
    cov_norm = npix / (npix - 1.0)
    ux, uy = _uniform(X, win), _uniform(Y, win)
    uxx, uyy, uxy = _uniform(X * X, win), _uniform(Y * Y, win), _uniform(X * Y, win)
    vx = cov_norm * (uxx - ux * ux)
    vy = cov_norm * (uyy - uy * uy)
    vxy = cov_norm * (uxy - ux * uy)
    C1 = (0.01 * data_range) ** 2
    C2 = (0.03 * data_range) ** 2
    S = ((2 * ux * uy + C1) * (2 * vxy + C2)) / ((ux ** 2 + uy ** 2 + C1) * (vx + vy + C2))
    pad = (win - 1) // 2
    return S[:, pad:S.shape[1] - pad, pad:S.shape[2] - pad].mean(dim=(1, 2)).tolist()
