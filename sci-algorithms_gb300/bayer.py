"""Bayer (colour mosaic) GAP-TV / ADMM-TV on the GPU.

``gap_denoise_bayer`` and ``admm_denoise_bayer`` of
``PnP_SCI/python/pnp_sci_algo.py:20-476`` for ``denoiser='tv'``.  The
reference splits the mosaic into its four RGGB sub-lattices
(``[[0,0],[0,1],[1,0],[1,1]]``, ``:112``), projects each with its own mask
and Phi_sum, and denoises the nmask*4 sub-lattice frames with one
multichannel TV call -- every frame on its own -- so the loop is four
independent GAP (ADMM) problems of size H/2 x W/2 x nmask.  Here each is a
native ``Solver`` (projection + TV per iteration, one CUDA graph), and the
result is re-assembled into the mosaic on the device.

Behavioural difference, on purpose: the reference's ADMM variant reads the
multiplier ``ball`` before assigning it (``:400``) and cannot run; here the
multiplier starts at zero, as in ``admm_denoise`` (``:802``).
"""
import math

import torch

from . import _dev
from .metrics import frame_psnr_ssim
from .solver import Solver
from .utils import MaskOperator

BAYER = ((0, 0), (0, 1), (1, 0), (1, 1))


def _iters(iter_max, sigma):
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    return int(sum(iter_max))


def _channels(y_bayer, Phi_bayer, x0_bayer, X_orig):
    """Device planes of the four sub-lattices: (y_c, op_c, x0_c, orig_c)."""
    y = _dev.plane(y_bayer)
    phi = _dev.planar(Phi_bayer)              # (B, H, W)
    B, H, W = phi.shape
    if H % 2 or W % 2:
        raise ValueError("the Bayer mosaic needs even H and W")
    x0 = None if x0_bayer is None else _dev.planar(x0_bayer)
    orig = None if X_orig is None else _dev.planar(X_orig)
    out = []
    for b0, b1 in BAYER:
        phic = phi[:, b0::2, b1::2].contiguous()
        op = MaskOperator(phic.permute(1, 2, 0))
        out.append((y[b0::2, b1::2].contiguous(), op,
                    None if x0 is None else x0[:, b0::2, b1::2].contiguous(),
                    None if orig is None else orig[:, b0::2, b1::2].contiguous()))
    return out, (B, H, W), phi.device


def _solve(projmeth, y_bayer, Phi_bayer, iters, _lambda, tv_weight, tv_iter_max, eps,
           accelerate, gamma, x0_bayer, X_orig, want_iqa, use_graph, tvm):
    chans, (B, H, W), dev = _channels(y_bayer, Phi_bayer, x0_bayer, X_orig if want_iqa else None)
    x_bayer = torch.empty((B, H, W), dtype=torch.float32, device=dev)
    # the four sub-lattice problems are independent: one stream each, so
    # that their kernels fill each other's tails
    main = torch.cuda.current_stream()
    streams = [torch.cuda.Stream(device=dev) for _ in BAYER]
    solvers = []
    for st, ((b0, b1), (yc, op, x0c, oc)) in zip(streams, zip(BAYER, chans)):
        st.wait_stream(main)
        with torch.cuda.stream(st):
            s = Solver(op, projmeth, iters, _lambda, tv_weight, tv_iter_max, eps, accelerate,
                       gamma, use_graph=use_graph, tvm=tvm)
            xc = s.run(yc, x0=x0c, orig=oc)
            x_bayer[:, b0::2, b1::2] = xc
        solvers.append((s, oc))
    sq = None
    for st, (s, oc) in zip(streams, solvers):
        main.wait_stream(st)
        if oc is not None:
            sq = s.sqerr.clone() if sq is None else sq + s.sqerr
    mse = [] if sq is None else [v / float(B * H * W) for v in sq.tolist()]
    return x_bayer, mse


def gap_denoise_bayer(y_bayer, Phi_bayer, _lambda=1, accelerate=True, denoiser='tv',
                      iter_max=50, noise_estimate=True, sigma=None, tv_weight=0.1,
                      tv_iter_max=5, multichannel=True, x0_bayer=None, X_orig=None,
                      model=None, show_iqa=True, eps=2.e-4, tvm='tv_chambolle',
                      use_graph=True):
    """GAP(-acc)-TV on a Bayer mosaic (``pnp_sci_algo.py:20-265``).

    y_bayer: H x W measurement; Phi_bayer: H x W x nmask full-resolution
    mask.  Returns ``(x_bayer, psnr_, ssim_, psnr_all)`` like the reference
    (x_bayer H x W x nmask; PSNR/SSIM per frame of the mosaic; PSNR of the
    mosaic per iteration, ``compare_psnr(..., data_range=1.)``)."""
    if str(denoiser).lower() != 'tv':
        raise ValueError("Unsupported denoiser {}!".format(denoiser))
    iters = _iters(iter_max, sigma)
    want_iqa = show_iqa and X_orig is not None
    x, mse = _solve("gap", y_bayer, Phi_bayer, iters, _lambda, tv_weight, tv_iter_max, eps,
                    accelerate, 0.0, x0_bayer, X_orig, want_iqa, use_graph, tvm)
    psnr_all = [10 * math.log10(1.0 / m) if m > 0 else math.inf for m in mse]
    psnr_, ssim_ = [], []
    if X_orig is not None:
        o = _dev.planar(X_orig)
        psnr_, ssim_ = frame_psnr_ssim(o, x)
    return _dev.unplanar(x, y_bayer), psnr_, ssim_, psnr_all


def admm_denoise_bayer(y_bayer, Phi_bayer, _lambda=1, gamma=0.01, denoiser='tv',
                       iter_max=50, noise_estimate=True, sigma=None, tv_weight=0.1,
                       tv_iter_max=5, multichannel=True, x0_bayer=None, X_orig=None,
                       model=None, show_iqa=True, eps=2.e-4, tvm='tv_chambolle',
                       use_graph=True):
    """ADMM-TV on a Bayer mosaic (``pnp_sci_algo.py:268-476``).  Returns
    ``(x_bayer, psnr_all)`` like the reference (PSNR of the mosaic per
    iteration, ``utils.psnr``)."""
    if str(denoiser).lower() != 'tv':
        raise ValueError("Unsupported denoiser {}!".format(denoiser))
    iters = _iters(iter_max, sigma)
    want_iqa = show_iqa and X_orig is not None
    x, mse = _solve("admm", y_bayer, Phi_bayer, iters, _lambda, tv_weight, tv_iter_max, eps,
                    True, gamma, x0_bayer, X_orig, want_iqa, use_graph, tvm)
    psnr_all = [100 if m == 0 else 20 * math.log10(1.0 / math.sqrt(m)) for m in mse]
    return _dev.unplanar(x, y_bayer), psnr_all
