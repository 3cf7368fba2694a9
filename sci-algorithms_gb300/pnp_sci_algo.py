"""GAP-TV / ADMM-TV drivers with the reference's call signatures.

Mirrors ``PnP_SCI/python/pnp_sci_algo.py``: ``admmdenoise_cacti``
(``:479-534``), ``gap_denoise`` (``:536-706``), ``admm_denoise``
(``:708-864``) and the legacy ``GAP_TV_rec`` / ``ADMM_TV_rec``
(``:866-907``), for ``denoiser='tv'``: ``tvm='tv_chambolle'`` (the
scikit-image TV of the Python reference) or one of the MATLAB twin's TV
denoisers (``tvm`` names of ``PnP_SCI/matlab/algorithms/gapdenoise.m:92-112``,
with gapdenoise's parameters and iteration counts); and for ``denoiser``
'ffdnet' / 'fastdvdnet' with ``model`` the network (``cnn.py``).

* When ``A`` / ``At`` are the bound methods of one ``MaskOperator`` (from
  ``make_ops(mask)``), the whole iteration loop runs natively
  (``sci_gap_tv`` / ``sci_admm_tv``: fused projection kernel + TV pipeline
  per iteration, replayed as a CUDA graph).
* Any other callables are used as plug-ins: they receive and return CUDA
  tensors (H x W x B views / H x W maps), the TV is the GPU kernel, and the
  projection arithmetic runs on the GPU.
* Extensions: ``tv_weight`` and ``_lambda`` may be per-iteration sequences;
  ``eps`` is the TV stop tolerance.
* Behavioural differences, on purpose: an unsupported ``projmeth`` or
  denoiser raises ``ValueError`` ('wavelet' and the colour / Bayer CNN
  variants are not built) (the reference prints and then fails on an
  unbound name, ``:518-519``), and TV errors propagate (the reference
  swallows ``TypeError``, ``:657-658``).

Outputs follow the measurement's kind: numpy in -> numpy float32 out; torch
in -> CUDA tensors out.
"""
import time

import numpy as np
import torch

from . import _dev
from .metrics import frame_psnr_ssim
from .solver import Solver
from .tv import TVM, tv_frames, tv_matlab_frames, tv_matlab_workspace, tv_workspace, tvm_kind
from .cassi import CassiOperator, CassiSolver
from .utils import MaskOperator, operator_of, psnr_from_mse, sum_sq_err


_CNN_DENOISERS = ("ffdnet", "fastdvdnet")


def _check_plugin(denoiser, tvm="tv_chambolle"):
    d = str(denoiser).lower()
    if d in _CNN_DENOISERS:
        return
    if d != "tv":
        raise ValueError("Unsupported denoiser {}!".format(denoiser))
    tvm_kind(tvm)  # raises ValueError for an unknown name


def _cnn_solve(projmeth, y, Phi_sum, A, At, iter_max, sigma, _lambda, gamma, accelerate,
               denoiser, model, x0, X_orig, show_iqa, precision):
    from .joint import cnn_denoise
    return cnn_denoise(projmeth, y, Phi_sum, A, At, iter_max, sigma, _lambda=_lambda,
                       gamma=gamma, accelerate=accelerate, denoiser=denoiser, model=model,
                       x0=x0, X_orig=X_orig if show_iqa else None, precision=precision)


def _total_iters(iter_max, sigma):
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    return int(sum(iter_max))


def _metrics(x_planar, X_orig, like):
    if X_orig is None:
        return [], []
    o = _dev.planar(X_orig)
    return frame_psnr_ssim(o, x_planar)


def _solve(projmeth, y, Phi_sum, A, At, iters, _lambda, tv_weight, tv_iter_max, eps,
           accelerate, gamma, x0, X_orig, show_iqa, use_graph, tvm="tv_chambolle"):
    """Shared body of gap_denoise / admm_denoise (native or plug-in)."""
    op = operator_of(A, At)
    y_d = _dev.plane(y)
    ps_d = _dev.plane(Phi_sum)
    want_iqa = show_iqa and X_orig is not None
    if isinstance(op, CassiOperator) and tvm != "tv_chambolle":
        raise ValueError("the spectral (CASSI) solver runs the scikit-image TV only")
    if isinstance(op, CassiOperator) and projmeth == "gap":
        solver = CassiSolver(op, iters, _lambda, tv_weight, tv_iter_max, eps, accelerate,
                             use_graph=use_graph)
        x0_d = None if x0 is None else _dev.planar(x0)
        orig_d = _dev.planar(X_orig) if want_iqa else None
        x = solver.run(y_d, x0=x0_d, phisum=ps_d, orig=orig_d)
        return x, (solver.psnr_all() if want_iqa else [])
    if isinstance(op, MaskOperator):
        solver = Solver(op, projmeth, iters, _lambda, tv_weight, tv_iter_max, eps, accelerate,
                        gamma, use_graph=use_graph, tvm=tvm)
        x0_d = None if x0 is None else _dev.planar(x0)
        orig_d = _dev.planar(X_orig) if want_iqa else None
        x = solver.run(y_d, x0=x0_d, phisum=ps_d, orig=orig_d)
        psnr_all = solver.psnr_all() if want_iqa else []
        return x, psnr_all
    if not (callable(A) and callable(At)):
        raise TypeError("A and At must be callables (or make_ops(mask))")
    return _solve_plugin(projmeth, y_d, ps_d, A, At, iters, _lambda, tv_weight, tv_iter_max,
                         eps, accelerate, gamma, x0, X_orig if want_iqa else None, tvm)


def _solve_plugin(projmeth, y, ps, A, At, iters, _lambda, tv_weight, tv_iter_max, eps,
                  accelerate, gamma, x0, X_orig, tvm="tv_chambolle"):
    """Iteration loop with foreign A / At callables (CUDA tensors in/out)."""
    lam = _dev.schedule(_lambda, iters)
    wts = _dev.schedule(tv_weight, iters)
    kind = tvm_kind(tvm)

    def fwd(xp):
        return _dev.plane(A(xp.permute(1, 2, 0)))

    def adj(r):
        return _dev.planar(At(r))

    x = adj(y) if x0 is None else _dev.planar(x0)
    B, H, W = x.shape
    if kind:
        _, param, tv_iters = TVM[tvm]
        ws = tv_matlab_workspace(kind, B, H, W, tv_iters, x.device)

    def denoise(v, k):
        if kind:
            return tv_matlab_frames(v, kind, param(float(wts[k])), tv_iters, workspace=ws)
        return tv_frames(v, float(wts[k]), tv_iter_max, eps, workspace=ws)

    if not kind:
        ws = tv_workspace(B, H, W, tv_iter_max, x.device)
    orig = None if X_orig is None else _dev.planar(X_orig)
    psnr_all = []
    if projmeth == "gap":
        y1 = torch.zeros_like(y)
        for k in range(iters):
            yb = fwd(x)
            if accelerate:
                y1 = y1 + (y - yb)
                xp = x + float(lam[k]) * adj((y1 - yb) / ps)
            else:
                xp = x + float(lam[k]) * adj((y - yb) / ps)
            x = denoise(xp.contiguous(), k)
            if orig is not None:
                psnr_all.append(psnr_from_mse(sum_sq_err(orig, x) / x.numel()))
        return x, psnr_all
    theta = x
    b = torch.zeros_like(x)
    for k in range(iters):
        t = theta + b
        yb = fwd(t)
        x = t + float(lam[k]) * adj((y - yb) / (ps + gamma))
        v = (x - b).contiguous()
        theta = denoise(v, k)
        b = theta - v  # b - (x - theta) = theta - (x - b)
        if orig is not None:
            psnr_all.append(psnr_from_mse(sum_sq_err(orig, x.contiguous()) / x.numel()))
    return x, psnr_all


def gap_denoise(y, Phi_sum, A, At, _lambda=1, accelerate=True, denoiser='tv', iter_max=50,
                noise_estimate=False, sigma=None, tv_weight=0.1, tv_iter_max=5,
                multichannel=True, x0=None, X_orig=None, model=None, show_iqa=True,
                tvm='tv_chambolle', eps=2.e-4, use_graph=True, precision=None):
    """GAP(-acc) with the TV denoiser (``pnp_sci_algo.py:536-706``), or
    with FFDNet / FastDVDnet (``denoiser`` 'ffdnet' / 'fastdvdnet', ``model``
    the network, ``sigma`` the per-stage noise levels, ``:667-670``).

    Returns ``(x, psnr_, ssim_, psnr_all)`` like the reference.
    """
    _check_plugin(denoiser, tvm)
    if str(denoiser).lower() in _CNN_DENOISERS:
        x, psnr_all = _cnn_solve("gap", y, Phi_sum, A, At, iter_max, sigma, _lambda, 0.0,
                                 accelerate, denoiser, model, x0, X_orig, show_iqa, precision)
        psnr_, ssim_ = _metrics(x, X_orig, y)
        return _dev.unplanar(x, y), psnr_, ssim_, psnr_all
    iters = _total_iters(iter_max, sigma)
    x, psnr_all = _solve("gap", y, Phi_sum, A, At, iters, _lambda, tv_weight, tv_iter_max, eps,
                         accelerate, 0.0, x0, X_orig, show_iqa, use_graph, tvm)
    psnr_, ssim_ = _metrics(x, X_orig, y)
    return _dev.unplanar(x, y), psnr_, ssim_, psnr_all


def admm_denoise(y, Phi_sum, A, At, _lambda=1, gamma=0.01, denoiser='tv', iter_max=50,
                 noise_estimate=False, sigma=None, tv_weight=0.1, tv_iter_max=5,
                 multichannel=True, x0=None, model=None, X_orig=None, show_iqa=True,
                 tvm='tv_chambolle', eps=2.e-4, use_graph=True, precision=None):
    """ADMM with the TV denoiser (``pnp_sci_algo.py:708-864``) or FFDNet /
    FastDVDnet (``:822-825``); returns ``(x, psnr_, ssim_, psnr_all)``."""
    _check_plugin(denoiser, tvm)
    if str(denoiser).lower() in _CNN_DENOISERS:
        x, psnr_all = _cnn_solve("admm", y, Phi_sum, A, At, iter_max, sigma, _lambda, gamma,
                                 True, denoiser, model, x0, X_orig, show_iqa, precision)
        psnr_, ssim_ = _metrics(x, X_orig, y)
        return _dev.unplanar(x, y), psnr_, ssim_, psnr_all
    iters = _total_iters(iter_max, sigma)
    x, psnr_all = _solve("admm", y, Phi_sum, A, At, iters, _lambda, tv_weight, tv_iter_max,
                         eps, True, gamma, x0, X_orig, show_iqa, use_graph, tvm)
    psnr_, ssim_ = _metrics(x, X_orig, y)
    return _dev.unplanar(x, y), psnr_, ssim_, psnr_all


def _flip(maskdirection, k):
    m = maskdirection.lower()
    return (m == 'updown' and k % 2 == 1) or (m == 'downup' and k % 2 == 0)


def admmdenoise_cacti(meas, mask, A, At, projmeth='admm', v0=None, orig=None, iframe=0,
                      nframe=1, MAXB=1., maskdirection='plain', **args):
    """Frame-block driver (``pnp_sci_algo.py:479-534``).

    meas: H x W x F measurements; mask: H x W x B; orig: H x W x (B F).
    Returns ``(x_, t_, psnr_, ssim_, psnrall_)``; x_ is float32.
    """
    if projmeth.lower() not in ('admm', 'gap'):
        raise ValueError('Unsupported projection method %s' % projmeth.upper())
    torch_in = _dev.is_torch(meas)
    nmask = mask.shape[-1]
    op = operator_of(A, At)
    if op is not None:
        mask_sum = op.phisum
    else:
        msk = _dev.planar(mask)
        mask_sum = msk.sum(dim=0)
        mask_sum = torch.where(mask_sum == 0, torch.ones_like(mask_sum), mask_sum)
    psnr_, ssim_, psnrall_ = [], [], []
    x_dev = None  # the H x W x (B nframe) result, assembled on the device
    # the measurements and the ground truth go to the device once; the
    # blocks are sliced there (host-side strided slices of H x W x F arrays
    # cost more than the copies)
    meas_d = _dev.stack(meas)
    orig_d = None if orig is None else _dev.stack(orig)
    begin = time.time()
    t_ = 0.0
    for kf in range(nframe):
        k = kf + iframe
        meas_k = meas_d[..., k] / MAXB  # block results stay on the device
        orig_k = None if orig_d is None else orig_d[..., k * nmask:(k + 1) * nmask] / MAXB
        v0_k = None
        if v0 is not None:
            v0_k = v0[:, :, kf * nmask:(kf + 1) * nmask]
            if _flip(maskdirection, k):
                v0_k = v0_k.flip(-1) if _dev.is_torch(v0_k) else v0_k[..., ::-1]
        fn = admm_denoise if projmeth.lower() == 'admm' else gap_denoise
        x_k, psnr_k, ssim_k, psnrall_k = fn(meas_k, mask_sum, A, At, x0=v0_k, X_orig=orig_k,
                                            **args)
        if _flip(maskdirection, k):
            x_k = x_k.flip(-1)
            psnr_k, ssim_k, psnrall_k = psnr_k[::-1], ssim_k[::-1], psnrall_k[::-1]
        if x_dev is None:
            x_dev = torch.empty((*x_k.shape[:-1], nmask * nframe), dtype=torch.float32,
                                device=x_k.device)
        x_dev[..., kf * nmask:(kf + 1) * nmask] = x_k
        torch.cuda.synchronize()
        t_ = time.time() - begin
        psnr_.extend(psnr_k)
        ssim_.extend(ssim_k)
        psnrall_.append(psnrall_k)
    if torch_in:
        return x_dev, t_, psnr_, ssim_, psnrall_
    # one copy of the whole result into page-locked host memory
    x_host = torch.empty(x_dev.shape, dtype=torch.float32, pin_memory=True)
    x_host.copy_(x_dev)
    return x_host.numpy(), t_, psnr_, ssim_, psnrall_


# ------------------------------------------------------------- legacy loops
def GAP_TV_rec(y, Phi, A, At, Phi_sum, maxiter, step_size, weight, row, col, ColT, X_ori,
               tv_n_iter=30):
    """``pnp_sci_algo.py:866-882``: GAP-acc with TV n_iter_max=30 from At(y).

    A / At are the two-argument operators (``A_``, ``At_``); the mask ``Phi``
    is bound here, so the native loop runs.
    """
    op = MaskOperator(Phi)
    s = Solver(op, "gap", int(maxiter), float(step_size), float(weight), tv_n_iter,
               accelerate=True)
    x = s.run(_dev.plane(y), phisum=_dev.plane(Phi_sum))
    return _dev.unplanar(x, y)


def ADMM_TV_rec(y, Phi, A, At, Phi_sum, maxiter, step_size, weight, row, col, ColT, eta,
                X_ori, tv_n_iter=30):
    """``pnp_sci_algo.py:884-907``: ADMM-TV with weight *= 0.999 and
    eta *= 0.998 after every iteration (``:898-899``); returns v."""
    n = int(maxiter)
    w = [float(weight)]
    g = [float(eta)]
    for _ in range(n - 1):
        w.append(0.999 * w[-1])
        g.append(0.998 * g[-1])
    op = MaskOperator(Phi)
    s = Solver(op, "admm", n, float(step_size), np.array(w), tv_n_iter, gammas=np.array(g))
    x = s.run(_dev.plane(y), phisum=_dev.plane(Phi_sum))
    return _dev.unplanar(x, y)
