"""Joint TV + CNN reconstruction (``PnP_SCI/python/joint_pnp_sci_algo.py``).

The reference runs, per coded-frame block, a first period of TV-only GAP or
ADMM iterations and a second period in which every iteration applies the TV
and then a CNN denoiser (FFDNet or FastDVDnet) at the stage's noise level
(``gap_joint_denoise`` / ``admm_joint_denoise``, ``:81-116``; the second
period is ``gap_multistep_denoise`` ``:309-499`` / ``admm_multistep_denoise``
``:118-307``).  The ADMM loops clip theta to [0, 1] after the denoiser.

Here the projections and the TV are this library's kernels on device
buffers.  ``model`` is the network the reference passes to
``ffdnet_vdenoiser(x, nsig, model)`` / ``fastdvdnet_denoiser(x, nsig, model,
gray=True)``: an FFDNet / FastDVDnet built by this package's classes or by
the reference's (converted on first use), run by ``cnn.CnnEngine`` over the
whole frame stack at once; any callable taking a planar (frames, H, W)
float32 CUDA tensor and the stage's ``nsig`` is accepted as well.
``denoiser`` is 'tv+ffdnet' or 'tv+fastdvdnet'; ``precision`` ('fp32',
'tf32', 'bf16') selects the network's arithmetic.  The TV is the
scikit-image Chambolle.
"""
import time

import torch

from . import _dev
from ._lib import call
from .metrics import frame_psnr_ssim
from .pnp_sci_algo import gap_denoise
from .tv import tv_frames, tv_workspace
from .utils import MaskOperator, operator_of, psnr_from_mse, sum_sq_err

_CNN = ("tv+ffdnet", "tv+fastdvdnet")


def _stages(iter_max, sigma):
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    return list(zip(iter_max, sigma))


class _Ops:
    """Projection steps on device buffers: the native kernels for a
    MaskOperator, the callables otherwise."""

    def __init__(self, A, At, y, ps):
        self.op = operator_of(A, At)
        self.A, self.At = A, At
        self.y, self.ps = y, ps
        self.native = isinstance(self.op, MaskOperator)

    def fwd(self, xp):
        return _dev.plane(self.A(xp.permute(1, 2, 0)))

    def adj(self, r):
        return _dev.planar(self.At(r))

    def x0(self):
        return self.adj(self.y)

    def gap(self, x, y1, lam, accelerate):
        """x + lam At((y1 - A x) / Phi_sum) (y1 += y - A x) or the plain GAP."""
        if self.native:
            op = self.op
            out = torch.empty_like(x)
            call("sci_proj_gap", x.data_ptr(), None if op.bits is not None else op.phi.data_ptr(),
                 _dev.ptr(op.bits), self.y.data_ptr(), _dev.ptr(y1), self.ps.data_ptr(),
                 out.data_ptr(), float(lam), int(accelerate), op.B, op.H, op.W,
                 _dev.stream_handle())
            return out
        yb = self.fwd(x)
        if accelerate:
            y1 += self.y - yb
            return x + lam * self.adj((y1 - yb) / self.ps)
        return x + lam * self.adj((self.y - yb) / self.ps)

    def admm(self, theta, b, lam, gamma):
        """(x, v) with x = theta + b + lam At((y - A(theta + b)) / (Phi_sum +
        gamma)) and v = x - b."""
        if self.native:
            op = self.op
            x = torch.empty_like(theta)
            v = torch.empty_like(theta)
            call("sci_proj_admm", theta.data_ptr(), b.data_ptr(),
                 None if op.bits is not None else op.phi.data_ptr(), _dev.ptr(op.bits),
                 self.y.data_ptr(), self.ps.data_ptr(), v.data_ptr(), x.data_ptr(), float(lam),
                 float(gamma), op.B, op.H, op.W, _dev.stream_handle())
            return x, v
        t = theta + b
        x = t + lam * self.adj((self.y - self.fwd(t)) / (self.ps + gamma))
        return x, (x - b).contiguous()


def _metrics(x, X_orig):
    if X_orig is None:
        return [], []
    o = _dev.planar(X_orig)
    return frame_psnr_ssim(o, x)


def cnn_step(denoiser, model, precision=None):
    """(x_planar, nsig, clip) -> denoised planar stack for a CNN denoiser
    name ('ffdnet' / 'fastdvdnet', with or without 'tv+').  ``model`` is an
    FFDNet / FastDVDnet network (this package's or the reference's classes;
    run by the batched CnnEngine) or any callable (x_planar, nsig) ->
    x_planar."""
    d = str(denoiser).lower()
    kind = "ffdnet" if d.endswith("ffdnet") and "fastdvd" not in d else "fastdvdnet"
    if isinstance(model, torch.nn.Module):
        from .cnn import engine_for
        eng = engine_for(model, kind, precision)
        return lambda x, nsig, clip: eng(x, nsig, clip)
    if not callable(model):
        raise TypeError("model must be an FFDNet / FastDVDnet network or a callable "
                        "(x_planar, nsig) -> x_planar")

    def run(x, nsig, clip):
        out = model(x, nsig).contiguous()
        return out.clamp(0, 1) if clip else out
    return run


def _loop(projmeth, y, Phi_sum, A, At, x0, stages, _lambda, gamma, accelerate, tv_weight,
          tv_iter_max, eps, X_orig, show_iqa, cnn, clip, tv=True):
    """One period: per iteration the projection, the TV (``tv``), the CNN
    step ``cnn`` (x, nsig, clip) at the stage's sigma when given, and (ADMM
    with ``clip``) the [0, 1] clip of theta."""
    y_d = _dev.plane(y)
    ps_d = _dev.plane(Phi_sum)
    ops = _Ops(A, At, y_d, ps_d)
    x = ops.x0() if x0 is None else _dev.planar(x0).clone()
    B, H, W = x.shape
    ws = tv_workspace(B, H, W, tv_iter_max, x.device) if tv else None
    orig = None if (X_orig is None or not show_iqa) else _dev.planar(X_orig)
    psnr_all = []

    def record(v):
        if orig is not None:
            psnr_all.append(psnr_from_mse(sum_sq_err(orig, v) / v.numel()))

    def denoise(v, nsig, clip_now):
        if tv:
            v = tv_frames(v, tv_weight, tv_iter_max, eps, workspace=ws)
        if cnn is not None:
            return cnn(v, nsig, clip_now)
        return v.clamp(0, 1) if clip_now else v

    if projmeth == "gap":
        y1 = torch.zeros_like(y_d)
        for iters, nsig in stages:
            for _ in range(int(iters)):
                xp = ops.gap(x, y1, _lambda, accelerate)
                x = denoise(xp.contiguous(), nsig, False)
                record(x)
        return x, psnr_all
    theta = x
    b = torch.zeros_like(x)
    for iters, nsig in stages:
        for _ in range(int(iters)):
            x, v = ops.admm(theta, b, _lambda, gamma)
            theta = denoise(v, nsig, clip)
            b = b - (x - theta)
            record(x)
    return x, psnr_all


# TV names each joint loop accepts (joint_pnp_sci_algo.py): the ADMM loops
# run the scikit-image Chambolle TV for all three (:296-303, :229-236); the
# GAP loops call denoise_tv_FGP_ITV3D / denoise_tv_cham_ITV2D, which the
# module never defines (:782-785, :433-436), so only tv_chambolle runs there.
_TVM_OK = {"gap": ("tv_chambolle",), "admm": ("tv_chambolle", "ITV3D_FGP", "ITV2D_cham")}


def _check(denoiser, tvm, model, cnn, projmeth="gap"):
    if tvm == "tv_bregman":
        raise ValueError("tvm='tv_bregman' (scikit-image's split-Bregman TV) is not built")
    if tvm not in _TVM_OK[projmeth]:
        raise ValueError("the joint %s loops run tvm in %s" % (projmeth, _TVM_OK[projmeth]))
    if cnn:
        if str(denoiser).lower() not in _CNN:
            raise ValueError("Unsupported denoiser {}!".format(denoiser))
        if model is None or not (callable(model) or isinstance(model, torch.nn.Module)):
            raise TypeError("model must be an FFDNet / FastDVDnet network or a callable "
                            "(x_planar, nsig) -> x_planar")
    elif str(denoiser).lower() != "tv":
        raise ValueError("Unsupported denoiser {}!".format(denoiser))


def cnn_denoise(projmeth, y, Phi_sum, A, At, iter_max, sigma, _lambda=1, gamma=0.0,
                accelerate=True, denoiser='ffdnet', model=None, x0=None, X_orig=None,
                show_iqa=True, precision=None):
    """The CNN-denoiser branches of pnp_sci_algo.py's gap_denoise /
    admm_denoise (``:667-670``, ``:822-825``): per iteration the projection
    and the network at the stage's sigma; returns (x_planar, psnr_all)."""
    if model is None:
        raise ValueError("denoiser %r needs model= (an FFDNet / FastDVDnet network; the "
                         "trained weights are not part of the reference tree)" % denoiser)
    step = cnn_step(denoiser, model, precision)
    return _loop(projmeth, y, Phi_sum, A, At, x0, _stages(iter_max, sigma), _lambda, gamma,
                 accelerate, 0.1, 1, 0.0, X_orig, show_iqa, step, False, tv=False)


def gap_multistep_denoise(y, Phi_sum, A, At, _lambda=1, gamma=None, accelerate=True,
                          denoiser='tv+ffdnet', iter_max=50, noise_estimate=False, sigma=None,
                          tv_weight=0.1, tv_iter_max=5, multichannel=True, x0=None,
                          X_orig=None, model=None, show_iqa=True, tvm='tv_chambolle',
                          eps=2.e-4, precision=None):
    """GAP with TV then CNN per iteration (joint_pnp_sci_algo.py:309-499).
    Returns ``(x, psnr_, ssim_, psnr_all)`` (x like y: numpy or torch)."""
    _check(denoiser, tvm, model, True, "gap")
    x, pa = _loop("gap", y, Phi_sum, A, At, x0, _stages(iter_max, sigma), _lambda, 0.0,
                  accelerate, tv_weight, tv_iter_max, eps, X_orig, show_iqa,
                  cnn_step(denoiser, model, precision), False)
    p, s = _metrics(x, X_orig)
    return _dev.unplanar(x, y), p, s, pa


def admm_multistep_denoise(y, Phi_sum, A, At, _lambda=1, gamma=0.0, accelerate=None,
                           denoiser='tv+ffdnet', iter_max=50, noise_estimate=False, sigma=None,
                           tv_weight=0.1, tv_iter_max=5, multichannel=True, x0=None, model=None,
                           X_orig=None, show_iqa=True, tvm='tv_chambolle', eps=2.e-4,
                           precision=None):
    """ADMM with theta = clip(CNN(TV(x - b))) per iteration
    (joint_pnp_sci_algo.py:118-307).  Returns ``(x, psnr_, ssim_, psnr_all)``."""
    _check(denoiser, tvm, model, True, "admm")
    x, pa = _loop("admm", y, Phi_sum, A, At, x0, _stages(iter_max, sigma), _lambda, gamma,
                  True, tv_weight, tv_iter_max, eps, X_orig, show_iqa,
                  cnn_step(denoiser, model, precision), True)
    p, s = _metrics(x, X_orig)
    return _dev.unplanar(x, y), p, s, pa


def _admm_tv_clip(y, Phi_sum, A, At, x0, iter_max, sigma, _lambda=1, gamma=0.0, tv_weight=0.1,
                  tv_iter_max=5, X_orig=None, show_iqa=True, eps=2.e-4, **_):
    """The first ADMM period: joint_pnp_sci_algo.py's admm_denoise
    (:502-664, denoiser='tv'), theta clipped to [0, 1]."""
    x, _ = _loop("admm", y, Phi_sum, A, At, x0, _stages(iter_max, sigma), _lambda, gamma, True,
                 tv_weight, tv_iter_max, eps, X_orig, False, None, True)
    return x


def gap_joint_denoise(y, Phi_sum, A, At, x0=None, X_orig=None, denoiser='tv+ffdnet',
                      iter_max1=50, iter_max2=50, sigma1=None, sigma2=None, **args):
    """TV-only GAP for ``iter_max1`` iterations, then TV + CNN for
    ``iter_max2`` (joint_pnp_sci_algo.py:100-116)."""
    model = args.pop("model", None)
    _check(denoiser, args.get("tvm", "tv_chambolle"), model, True, "gap")
    first = {k: v for k, v in args.items() if k not in ("gamma", "show_iqa", "precision")}
    y_d = _dev.plane(y)  # both periods on device buffers
    x, _, _, _ = gap_denoise(y_d, Phi_sum, A, At, x0=x0, X_orig=X_orig, denoiser='tv',
                             iter_max=iter_max1, sigma=sigma1, show_iqa=False, **first)
    x, p, s, pa = gap_multistep_denoise(y_d, Phi_sum, A, At, x0=x, X_orig=X_orig,
                                        denoiser=denoiser, iter_max=iter_max2, sigma=sigma2,
                                        model=model, **args)
    return _dev.unplanar(_dev.planar(x), y), p, s, pa


def admm_joint_denoise(y, Phi_sum, A, At, x0=None, X_orig=None, denoiser='tv+ffdnet',
                       iter_max1=50, iter_max2=50, sigma1=None, sigma2=None, **args):
    """TV-only ADMM (theta clipped) for ``iter_max1`` iterations, then TV +
    CNN for ``iter_max2`` (joint_pnp_sci_algo.py:81-97)."""
    model = args.pop("model", None)
    _check(denoiser, args.get("tvm", "tv_chambolle"), model, True, "admm")
    y_d = _dev.plane(y)
    x = _admm_tv_clip(y_d, Phi_sum, A, At, x0, iter_max1, sigma1, **args)
    x, p, s, pa = admm_multistep_denoise(y_d, Phi_sum, A, At, x0=x.permute(1, 2, 0),
                                         X_orig=X_orig, denoiser=denoiser, iter_max=iter_max2,
                                         sigma=sigma2, model=model, **args)
    return _dev.unplanar(_dev.planar(x), y), p, s, pa


def joint_admmdenoise_cacti(meas, mask, A, At, projmeth='admm', v0=None, orig=None, iframe=0,
                            nframe=1, MAXB=1., maskdirection='plain', denoiser='tv',
                            iter_max1=50, iter_max2=50, sigma1=None, sigma2=None, **args):
    """Frame-block driver of the joint loops (joint_pnp_sci_algo.py:20-59).
    meas: H x W x F; mask: H x W x B; orig: H x W x (B F); ``model`` (in
    ``args``) is the CNN plug-in.  Returns ``(x_, t_, psnr_, ssim_,
    psnrall_)``."""
    if projmeth.lower() not in ('admm', 'gap'):
        raise ValueError('Unsupported projection method %s' % projmeth.upper())
    nmask = mask.shape[-1]
    op = operator_of(A, At)
    if op is not None:
        mask_sum = op.phisum
    else:
        msk = _dev.planar(mask)
        mask_sum = msk.sum(dim=0)
        mask_sum = torch.where(mask_sum == 0, torch.ones_like(mask_sum), mask_sum)
    fn = admm_joint_denoise if projmeth.lower() == 'admm' else gap_joint_denoise
    torch_in = _dev.is_torch(meas)
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
        flip = (maskdirection.lower() == 'updown' and k % 2 == 1) or \
               (maskdirection.lower() == 'downup' and k % 2 == 0)
        meas_k = meas_d[..., k] / MAXB  # block results stay on the device
        orig_k = None if orig_d is None else orig_d[..., k * nmask:(k + 1) * nmask] / MAXB
        v0_k = None
        if v0 is not None:
            v0_k = v0[:, :, kf * nmask:(kf + 1) * nmask]
            if flip:
                v0_k = v0_k.flip(-1) if _dev.is_torch(v0_k) else v0_k[..., ::-1]
        x_k, psnr_k, ssim_k, psnrall_k = fn(meas_k, mask_sum, A, At, x0=v0_k, X_orig=orig_k,
                                            denoiser=denoiser, iter_max1=iter_max1,
                                            iter_max2=iter_max2, sigma1=sigma1, sigma2=sigma2,
                                            **dict(args))
        if flip:
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
        x_ = x_dev
    else:
        x_host = torch.empty(x_dev.shape, dtype=torch.float32, pin_memory=True)
        x_host.copy_(x_dev)
        x_ = x_host.numpy()
    return x_, t_, psnr_, ssim_, psnrall_
