"""CPU oracle: the reference's numpy GAP/ADMM path, restated.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, and only as the checker.

Each function restates one reference function with the same numpy operation
order, so that a float64 run is bit-identical to the reference's own code.
That identity is pinned: ``tests/golden/make_golden.py`` imports the
reference modules themselves (``PnP_SCI/python/utils.py``,
``PnP_SCI/python/pnp_sci_algo.py``) with the third-party imports replaced by
``oracle.tv_chambolle`` and the metric restatements below, runs them on
seeded inputs and stores the outputs; ``tests/test_oracle.py`` checks this
port against those fixtures bit for bit.

Extensions over the reference, used by the large configurations and marked
where they appear: ``tv_weight`` and ``_lambda`` may be per-iteration
sequences (a schedule); ``eps`` of the TV may be passed through.
"""
import math
import time

import numpy as np
from scipy.ndimage import uniform_filter

from . import cnn as _cnn
from .tv_chambolle import denoise_tv_chambolle


# ---------------------------------------------------------------- L1 operators
def A_(x, Phi):
    """``PnP_SCI/python/utils.py:10-15``: y = sum_b x[..., b] * Phi[..., b]."""
    return np.sum(x * Phi, axis=2)


def At_(y, Phi):
    """``PnP_SCI/python/utils.py:17-26``: x[..., b] = y * Phi[..., b]."""
    return np.multiply(np.repeat(y[:, :, np.newaxis], Phi.shape[2], axis=2), Phi)


def psnr(ref, img):
    """``PnP_SCI/python/utils.py:28-36`` (peak 1, returns 100 when equal)."""
    mse = np.mean((ref - img) ** 2)
    if mse == 0:
        return 100
    return 20 * math.log10(1.0 / math.sqrt(mse))


# ------------------------------------------------------- third-party metrics
def compare_psnr(im_true, im_test, data_range=None):
    """scikit-image 0.16 ``measure.compare_psnr``: 10 log10(R^2 / MSE).

    Called per frame at ``pnp_sci_algo.py:704`` and ``:862`` with
    ``data_range=1``.  The MSE is taken in float64.
    """
    im_true = np.asarray(im_true, dtype=np.float64)
    im_test = np.asarray(im_test, dtype=np.float64)
    err = np.mean(np.square(im_true - im_test), dtype=np.float64)
    return 10 * np.log10((data_range ** 2) / err)


def compare_ssim(X, Y, win_size=None, data_range=None, multichannel=False,
                 **_unused):
    """scikit-image 0.16 ``measure.compare_ssim`` with its default options.

    Wang et al. (2004) SSIM with a 7 x 7 uniform window
    (``scipy.ndimage.uniform_filter``, mode 'reflect'), sample covariance
    (N / (N - 1)), K1 = 0.01, K2 = 0.03, and the mean taken over the image
    cropped by (win_size - 1) // 2 on every side.  The reference calls it
    per frame with ``data_range=1`` (``pnp_sci_algo.py:705``, ``:863``).
    """
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    if multichannel:
        return float(np.mean([compare_ssim(X[..., c], Y[..., c], win_size,
                                           data_range) for c in range(X.shape[-1])]))
    win = 7 if win_size is None else win_size
    ndim = X.ndim
    npix = win ** ndim
    cov_norm = npix / (npix - 1.0)
    ux = uniform_filter(X, size=win)
    uy = uniform_filter(Y, size=win)
    uxx = uniform_filter(X * X, size=win)
    uyy = uniform_filter(Y * Y, size=win)
    uxy = uniform_filter(X * Y, size=win)
    vx = cov_norm * (uxx - ux * ux)
    vy = cov_norm * (uyy - uy * uy)
    vxy = cov_norm * (uxy - ux * uy)
    R = data_range
    C1 = (0.01 * R) ** 2
    C2 = (0.03 * R) ** 2
    A1, A2, B1, B2 = (2 * ux * uy + C1, 2 * vxy + C2,
                      ux ** 2 + uy ** 2 + C1, vx + vy + C2)
    S = (A1 * A2) / (B1 * B2)
    pad = (win - 1) // 2
    crop = tuple(slice(pad, s - pad) for s in S.shape)
    return float(S[crop].mean())


# ---------------------------------------------------------------- schedules
def _at(seq_or_scalar, k):
    """Value of a per-iteration schedule at iteration k (extension)."""
    if np.ndim(seq_or_scalar) == 0:
        return seq_or_scalar
    return seq_or_scalar[k]


def annealed_weights(w0, w1, n):
    """Geometric tv_weight schedule w_k = w0 (w1/w0)^(k/(n-1)).

    Extends the multiplicative annealing of ``ADMM_TV_rec``
    (``pnp_sci_algo.py:898``: ``weight = 0.999*weight`` per iteration) to
    fixed end points; used for the 2048 x 2048 x 24 configuration
    (0.2 -> 0.05 over 60 iterations).
    """
    if n == 1:
        return np.array([w0], dtype=np.float64)
    k = np.arange(n, dtype=np.float64)
    return w0 * (w1 / w0) ** (k / (n - 1))


# ---------------------------------------------------------------- L2 solvers
def _check_denoiser(denoiser, tvm):
    d = denoiser.lower()
    if d not in ('tv', 'ffdnet', 'fastdvdnet') or (d == 'tv' and tvm != 'tv_chambolle'):
        raise ValueError('oracle supports denoiser "tv" (tv_chambolle), "ffdnet", "fastdvdnet"')


def _denoise(x, denoiser, w, eps, tv_iter_max, multichannel, nsig, model, threads=1):
    """The denoiser switch of gap_denoise / admm_denoise (pnp_sci_algo.py:647-672)."""
    d = denoiser.lower()
    if d == 'ffdnet':
        return _cnn.ffdnet_vdenoiser(x, nsig, model)
    if d == 'fastdvdnet':
        return _cnn.fastdvdnet_denoiser(x, nsig, model, gray=True)
    return denoise_tv_chambolle(x, w, eps=eps, n_iter_max=tv_iter_max, multichannel=multichannel,
                                threads=threads)


def gap_iteration(y, y1, x, Phi_sum, A, At, lam, w, accelerate=True, denoiser='tv',
                  eps=2.e-4, tv_iter_max=5, multichannel=True, nsig=None, model=None,
                  threads=1, resid=None):
    """One iteration of ``gap_denoise``'s loop (``pnp_sci_algo.py:639-650``):
    the GAP (``:645``) or accelerated GAP (``:641-643``) projection, then the
    denoiser (its frames on ``threads`` threads).  Returns the new (x, y1).
    ``resid`` (a list) receives ||r||^2 of the projection's residual map
    r = (y1 - yb) / Phi_sum (or (y - yb) / Phi_sum), in float64."""
    yb = A(x)
    if accelerate:
        y1 = y1 + (y - yb)
        r = (y1 - yb) / Phi_sum
    else:
        r = (y - yb) / Phi_sum
    x = x + lam * (At(r))
    if resid is not None:
        resid.append(float(np.sum(np.asarray(r, np.float64) ** 2)))
    x = _denoise(x, denoiser, w, eps, tv_iter_max, multichannel, nsig, model, threads)
    return x, y1


def gap_denoise(y, Phi_sum, A, At, _lambda=1, accelerate=True,
                denoiser='tv', iter_max=50, noise_estimate=False, sigma=None,
                tv_weight=0.1, tv_iter_max=5, multichannel=True, x0=None,
                X_orig=None, model=None, show_iqa=True, tvm='tv_chambolle',
                eps=2.e-4, verbose=False, resid=None):
    """``PnP_SCI/python/pnp_sci_algo.py:536-706``.

    GAP (``:645``) or accelerated GAP (``:641-643``) projection, then the
    Chambolle TV (``:650``) or, for ``denoiser`` 'ffdnet' / 'fastdvdnet'
    (``:667-670``), the CNN of ``oracle.cnn`` with ``model`` its parameter
    dict at the stage's sigma.  ``tv_weight`` / ``_lambda`` may also be
    sequences indexed by the global iteration (extension).
    """
    _check_denoiser(denoiser, tvm)
    if x0 is None:
        x0 = At(y)
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    y1 = np.zeros_like(y)
    x = x0
    psnr_all = []
    k = 0
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            x, y1 = gap_iteration(y, y1, x, Phi_sum, A, At, _at(_lambda, k), _at(tv_weight, k),
                                  accelerate, denoiser, eps, tv_iter_max, multichannel, nsig,
                                  model, resid=resid)
            if show_iqa and X_orig is not None:
                psnr_all.append(psnr(X_orig, x))
                if verbose and (k + 1) % 5 == 0:
                    print('  GAP-TV iteration {: 3d}, PSNR {:2.2f} dB.'.format(
                        k + 1, psnr_all[k]))
            k = k + 1
    psnr_, ssim_ = [], []
    nmask = x.shape[-1]
    if X_orig is not None:
        for imask in range(nmask):
            psnr_.append(compare_psnr(X_orig[..., imask], x[..., imask], data_range=1.))
            ssim_.append(compare_ssim(X_orig[..., imask], x[..., imask], data_range=1.,
                                      multichannel=x[..., imask].ndim > 2))
    return x, psnr_, ssim_, psnr_all


def admm_denoise(y, Phi_sum, A, At, _lambda=1, gamma=0.01,
                 denoiser='tv', iter_max=50, noise_estimate=False, sigma=None,
                 tv_weight=0.1, tv_iter_max=5, multichannel=True, x0=None,
                 model=None, X_orig=None, show_iqa=True, eps=2.e-4,
                 verbose=False, resid=None):
    """``PnP_SCI/python/pnp_sci_algo.py:708-864``.

    yb = A(theta + b); x = theta + b + lambda At((y - yb)/(Phi_sum + gamma))
    (``:808-809``); theta = TV(x - b) (``:812-813``) or the CNN of
    ``oracle.cnn`` (``:822-825``); b = b - (x - theta) (``:836``).
    Returns x, not theta (``:864``).  ``resid`` (a list) receives ||r||^2 of
    every iteration's residual map r = (y - yb) / (Phi_sum + gamma).
    """
    _check_denoiser(denoiser, 'tv_chambolle')
    if x0 is None:
        x0 = At(y)
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    x = x0
    theta = x0
    b = np.zeros_like(x0)
    psnr_all = []
    k = 0
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            lam = _at(_lambda, k)
            w = _at(tv_weight, k)
            yb = A(theta + b)
            r = (y - yb) / (Phi_sum + gamma)
            x = (theta + b) + lam * (At(r))
            if resid is not None:
                resid.append(float(np.sum(np.asarray(r, np.float64) ** 2)))
            theta = _denoise(x - b, denoiser, w, eps, tv_iter_max, multichannel, nsig, model)
            b = b - (x - theta)
            if show_iqa and X_orig is not None:
                psnr_all.append(psnr(X_orig, x))
                if verbose and (k + 1) % 5 == 0:
                    print('  ADMM-TV iteration {: 3d}, PSNR {:2.2f} dB.'.format(
                        k + 1, psnr_all[k]))
            k = k + 1
    psnr_, ssim_ = [], []
    nmask = x.shape[2]
    if X_orig is not None:
        for imask in range(nmask):
            psnr_.append(compare_psnr(X_orig[:, :, imask], x[:, :, imask], data_range=1.))
            ssim_.append(compare_ssim(X_orig[:, :, imask], x[:, :, imask], data_range=1.))
    return x, psnr_, ssim_, psnr_all


def admmdenoise_cacti(meas, mask, A, At, projmeth='admm', v0=None, orig=None,
                      iframe=0, nframe=1, MAXB=1., maskdirection='plain',
                      **args):
    """``PnP_SCI/python/pnp_sci_algo.py:479-534``: the frame-block driver.

    Phi_sum with zeros replaced by 1 (``:491-492``), per-block scaling by
    MAXB (``:501-503``), v0 flips for 'updown'/'downup' masks
    (``:506-510``, ``:521-527``).  An unknown ``projmeth`` raises
    ValueError (the reference only prints, ``:518-519``).
    """
    nmask = mask.shape[-1]
    mask_sum = np.sum(mask, axis=tuple(range(2, mask.ndim)))
    mask_sum[mask_sum == 0] = 1
    x_ = np.zeros((*mask.shape[:-1], nmask * nframe), dtype=np.float32)
    psnr_, ssim_, psnrall_ = [], [], []
    begin_time = time.time()
    orig_k = None
    for kf in range(nframe):
        if orig is not None:
            orig_k = orig[..., (kf + iframe) * nmask:(kf + iframe + 1) * nmask] / MAXB
        meas_k = meas[..., kf + iframe] / MAXB
        if v0 is None:
            v0_k = None
        else:
            v0_k = v0[:, :, kf * nmask:(kf + 1) * nmask]
            if (maskdirection.lower() == 'updown' and (kf + iframe) % 2 == 1) or \
               (maskdirection.lower() == 'downup' and (kf + iframe) % 2 == 0):
                v0_k = v0_k[..., ::-1]
        if projmeth.lower() == 'admm':
            x_k, psnr_k, ssim_k, psnrall_k = admm_denoise(
                meas_k, mask_sum, A, At, x0=v0_k, X_orig=orig_k, **args)
        elif projmeth.lower() == 'gap':
            x_k, psnr_k, ssim_k, psnrall_k = gap_denoise(
                meas_k, mask_sum, A, At, x0=v0_k, X_orig=orig_k, **args)
        else:
            raise ValueError('Unsupported projection method %s' % projmeth.upper())
        if (maskdirection.lower() == 'updown' and (kf + iframe) % 2 == 1) or \
           (maskdirection.lower() == 'downup' and (kf + iframe) % 2 == 0):
            x_k = x_k[..., ::-1]
            psnr_k = psnr_k[::-1]
            ssim_k = ssim_k[::-1]
            psnrall_k = psnrall_k[::-1]
        t_ = time.time() - begin_time
        x_[..., kf * nmask:(kf + 1) * nmask] = x_k
        psnr_.extend(psnr_k)
        ssim_.extend(ssim_k)
        psnrall_.append(psnrall_k)
    return x_, t_, psnr_, ssim_, psnrall_


# ------------------------------------------------------------- legacy loops
def GAP_TV_rec(y, Phi, A, At, Phi_sum, maxiter, step_size, weight, row, col,
               ColT, X_ori, tv_n_iter=30):
    """``PnP_SCI/python/pnp_sci_algo.py:866-882`` (two-argument A/At)."""
    y1 = np.zeros((row, col))
    f = At(y, Phi)
    for ni in range(maxiter):
        fb = A(f, Phi)
        y1 = y1 + (y - fb)
        f = f + np.multiply(step_size, At(np.divide(y1 - fb, Phi_sum), Phi))
        f = denoise_tv_chambolle(f, weight, n_iter_max=tv_n_iter, multichannel=True)
    return f


def ADMM_TV_rec(y, Phi, A, At, Phi_sum, maxiter, step_size, weight, row, col,
                ColT, eta, X_ori, tv_n_iter=30):
    """``PnP_SCI/python/pnp_sci_algo.py:884-907``; anneals weight *= 0.999
    and eta *= 0.998 every iteration (``:898-899``)."""
    theta = At(y, Phi)
    v = theta
    b = np.zeros((row, col, ColT))
    for ni in range(maxiter):
        yb = A(theta + b, Phi)
        v = (theta + b) + np.multiply(step_size, At(np.divide(y - yb, Phi_sum + eta), Phi))
        theta = denoise_tv_chambolle(v - b, weight, n_iter_max=tv_n_iter, multichannel=True)
        b = b - (v - theta)
        weight = 0.999 * weight
        eta = 0.998 * eta
    return v


# ---------------------------------------------------------------- Bayer loops
BAYER = [[0, 0], [0, 1], [1, 0], [1, 1]]  # pnp_sci_algo.py:112 (RGGB sub-lattices)


def _bayer_split(y_bayer, Phi_bayer, x0_bayer):
    """The channel set-up of pnp_sci_algo.py:120-140 / :353-379: float32
    sub-lattice measurements, masks, Phi_sum (zeros -> 1) and x0."""
    nrow, ncol, nmask = Phi_bayer.shape
    yall = np.zeros([nrow // 2, ncol // 2, 4], dtype=np.float32)
    Phiall = np.zeros([nrow // 2, ncol // 2, nmask, 4], dtype=np.float32)
    Phi_sumall = np.zeros([nrow // 2, ncol // 2, 4], dtype=np.float32)
    x0all = np.zeros([nrow // 2, ncol // 2, nmask, 4], dtype=np.float32)
    for ib, b in enumerate(BAYER):
        yall[..., ib] = y_bayer[b[0]::2, b[1]::2]
        Phiall[..., ib] = Phi_bayer[b[0]::2, b[1]::2]
        Phib_sum = np.sum(Phiall[..., ib], axis=2)
        Phib_sum[Phib_sum == 0] = 1
        Phi_sumall[..., ib] = Phib_sum
        if x0_bayer is None:
            x0all[..., ib] = At_(yall[..., ib], Phiall[..., ib])
        else:
            x0all[..., ib] = x0_bayer[b[0]::2, b[1]::2]
    return yall, Phiall, Phi_sumall, x0all


def _bayer_join(xall, like):
    x_bayer = np.zeros_like(like)
    for ib, b in enumerate(BAYER):
        x_bayer[b[0]::2, b[1]::2] = xall[..., ib]
    return x_bayer


def gap_denoise_bayer(y_bayer, Phi_bayer, _lambda=1, accelerate=True, denoiser='tv',
                      iter_max=50, noise_estimate=True, sigma=None, tv_weight=0.1,
                      tv_iter_max=5, multichannel=True, x0_bayer=None, X_orig=None,
                      model=None, show_iqa=True):
    """``PnP_SCI/python/pnp_sci_algo.py:20-265`` with ``denoiser='tv'``.

    Four independent GAP(-acc) projections on the sub-lattice channels
    (``:149-157``, in place on float32 arrays), then one Chambolle TV over
    the nmask*4 frames (``:161-165``).  PSNR per iteration on the
    re-assembled Bayer image (``:241-246``)."""
    if denoiser.lower() != 'tv':
        raise ValueError('oracle supports denoiser="tv"')
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    nrow, ncol, nmask = Phi_bayer.shape
    yall, Phiall, Phi_sumall, x0all = _bayer_split(y_bayer, Phi_bayer, x0_bayer)
    y1all = np.zeros_like(yall)
    xall = x0all
    psnr_all = []
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            for ib in range(4):
                yb = A_(xall[..., ib], Phiall[..., ib])
                if accelerate:
                    y1all[..., ib] += (yall[..., ib] - yb)
                    xall[..., ib] += _lambda * (At_((y1all[..., ib] - yb) / Phi_sumall[..., ib],
                                                    Phiall[..., ib]))
                else:
                    xall[..., ib] += _lambda * (At_((yall[..., ib] - yb) / Phi_sumall[..., ib],
                                                    Phiall[..., ib]))
            xall_vch = xall.reshape([nrow // 2, ncol // 2, nmask * 4])
            xall_vch = denoise_tv_chambolle(xall_vch, tv_weight, n_iter_max=tv_iter_max,
                                            multichannel=multichannel)
            xall = xall_vch.reshape([nrow // 2, ncol // 2, nmask, 4])
            if show_iqa and X_orig is not None:
                psnr_all.append(compare_psnr(X_orig, _bayer_join(xall, Phi_bayer),
                                             data_range=1.))
    x_bayer = _bayer_join(xall, Phi_bayer)
    psnr_, ssim_ = [], []
    if X_orig is not None:
        for imask in range(nmask):
            psnr_.append(compare_psnr(X_orig[:, :, imask], x_bayer[:, :, imask], data_range=1.))
            ssim_.append(compare_ssim(X_orig[:, :, imask], x_bayer[:, :, imask], data_range=1.))
    return x_bayer, psnr_, ssim_, psnr_all


def admm_denoise_bayer(y_bayer, Phi_bayer, _lambda=1, gamma=0.01, denoiser='tv',
                       iter_max=50, noise_estimate=True, sigma=None, tv_weight=0.1,
                       tv_iter_max=5, multichannel=True, x0_bayer=None, X_orig=None,
                       model=None, show_iqa=True):
    """``PnP_SCI/python/pnp_sci_algo.py:268-476`` with ``denoiser='tv'``.

    The reference reads the multiplier ``ball`` before assigning it
    (``:400``; it initialises ``b``, ``:389``), so it cannot run; this
    restatement starts ``ball`` at zero, as admm_denoise does (``:802``).
    Per iteration: four ADMM projections x = theta + b + lambda At((y -
    A(theta + b)) / (Phi_sum + gamma)) (``:399-401``), theta = TV(x - b)
    over the nmask*4 frames (``:407-410``), b = b - (x - theta) (``:442``).
    Returns the Bayer image of x and the PSNR per iteration."""
    if denoiser.lower() != 'tv':
        raise ValueError('oracle supports denoiser="tv"')
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    nrow, ncol, nmask = Phi_bayer.shape
    yall, Phiall, Phi_sumall, x0all = _bayer_split(y_bayer, Phi_bayer, x0_bayer)
    xall = x0all.copy()
    thetaall = x0all.copy()
    ball = np.zeros_like(x0all)
    psnr_all = []
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            for ib in range(4):
                yb = A_(thetaall[..., ib] + ball[..., ib], Phiall[..., ib])
                xall[..., ib] = thetaall[..., ib] + ball[..., ib] + _lambda * (
                    At_((yall[..., ib] - yb) / (Phi_sumall[..., ib] + gamma), Phiall[..., ib]))
            thetaall_vch = (xall - ball).reshape([nrow // 2, ncol // 2, nmask * 4])
            thetaall_vch = denoise_tv_chambolle(thetaall_vch, tv_weight,
                                                n_iter_max=tv_iter_max, multichannel=multichannel)
            thetaall = thetaall_vch.reshape([nrow // 2, ncol // 2, nmask, 4])
            ball = ball - (xall - thetaall)
            if show_iqa and X_orig is not None:
                psnr_all.append(psnr(X_orig, _bayer_join(xall, Phi_bayer)))
    return _bayer_join(xall, Phi_bayer), psnr_all


# ------------------------------------------------- joint TV + CNN loops
def box_blur(x):
    """The stand-in CNN of the joint fixtures: a 3 x 3 box blur of every
    frame with replicated edges (the FFDNet / FastDVDnet weights are not in
    the reference tree)."""
    x = np.asarray(x, np.float64)
    xp = np.pad(x, ((1, 1), (1, 1), (0, 0)), mode="edge")
    H, W = x.shape[:2]
    out = np.zeros_like(x)
    for di in range(3):
        for dj in range(3):
            out += xp[di:di + H, dj:dj + W]
    return out / 9.0


def cnn_stand_in(x, nsig, model=None, gray=True):
    """(x, nsig, model) -> x, the call shape of ffdnet_vdenoiser /
    fastdvdnet_denoiser; here the box blur."""
    return box_blur(x)


# PnP_SCI/python/joint_pnp_sci_algo.py.  `cnn(x, nsig, model)` stands where
# the reference calls ffdnet_vdenoiser(x, nsig, model) /
# fastdvdnet_denoiser(x, nsig, model, gray=True) (:243, :267, :442, :467).
def _tv_step(x, tv_weight, tv_iter_max, multichannel, tvm):
    if tvm not in ('tv_chambolle', 'ITV3D_FGP', 'ITV2D_cham'):
        raise ValueError('oracle supports the tv_chambolle denoiser')
    return denoise_tv_chambolle(x, tv_weight, n_iter_max=tv_iter_max, multichannel=multichannel)


def joint_admm_denoise(y, Phi_sum, A, At, _lambda=1, gamma=0.0, denoiser='tv', iter_max=50,
                       sigma=None, tv_weight=0.1, tv_iter_max=5, multichannel=True, x0=None,
                       X_orig=None, show_iqa=True, tvm='tv_chambolle', **_):
    """``joint_pnp_sci_algo.py:502-664`` (denoiser='tv'): admm_denoise with
    theta clipped to [0, 1] after the denoiser (``:640``)."""
    if x0 is None:
        x0 = At(y)
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    x = x0
    theta = x0
    b = np.zeros_like(x0)
    psnr_all = []
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            yb = A(theta + b)
            x = (theta + b) + _lambda * (At((y - yb) / (Phi_sum + gamma)))
            theta = _tv_step(x - b, tv_weight, tv_iter_max, multichannel, tvm)
            theta = np.clip(theta, 0, 1)
            b = b - (x - theta)
            if show_iqa and X_orig is not None:
                psnr_all.append(psnr(X_orig, x))
    psnr_, ssim_ = _frame_metrics(X_orig, x)
    return x, psnr_, ssim_, psnr_all


def _frame_metrics(X_orig, x):
    psnr_, ssim_ = [], []
    if X_orig is not None:
        for imask in range(x.shape[2]):
            psnr_.append(compare_psnr(X_orig[:, :, imask], x[:, :, imask], data_range=1.))
            ssim_.append(compare_ssim(X_orig[:, :, imask], x[:, :, imask], data_range=1.))
    return psnr_, ssim_


def gap_multistep_denoise(y, Phi_sum, A, At, cnn, _lambda=1, accelerate=True,
                          denoiser='tv+ffdnet', iter_max=50, sigma=None, tv_weight=0.1,
                          tv_iter_max=5, multichannel=True, x0=None, X_orig=None, model=None,
                          show_iqa=True, tvm='tv_chambolle', **_):
    """``joint_pnp_sci_algo.py:309-499``: per iteration the GAP(-acc)
    projection, the TV, then the CNN at this stage's sigma."""
    if x0 is None:
        x0 = At(y)
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    y1 = np.zeros_like(y)
    x = x0
    psnr_all = []
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            yb = A(x)
            if accelerate:
                y1 = y1 + (y - yb)
                x = x + _lambda * (At((y1 - yb) / Phi_sum))
            else:
                x = x + _lambda * (At((y - yb) / Phi_sum))
            x = _tv_step(x, tv_weight, tv_iter_max, multichannel, tvm)
            x = cnn(x, nsig, model)
            if show_iqa and X_orig is not None:
                psnr_all.append(psnr(X_orig, x))
    psnr_, ssim_ = _frame_metrics(X_orig, x)
    return x, psnr_, ssim_, psnr_all


def admm_multistep_denoise(y, Phi_sum, A, At, cnn, _lambda=1, gamma=0.0,
                           denoiser='tv+ffdnet', iter_max=50, sigma=None, tv_weight=0.1,
                           tv_iter_max=5, multichannel=True, x0=None, X_orig=None, model=None,
                           show_iqa=True, tvm='tv_chambolle', **_):
    """``joint_pnp_sci_algo.py:118-307``: per iteration the ADMM projection,
    theta = CNN(TV(x - b)), clipped to [0, 1] (``:289``), b -= x - theta."""
    if x0 is None:
        x0 = At(y)
    if not isinstance(sigma, list):
        sigma = [sigma]
    if not isinstance(iter_max, list):
        iter_max = [iter_max] * len(sigma)
    x = x0
    theta = x0
    b = np.zeros_like(x0)
    psnr_all = []
    for idx, nsig in enumerate(sigma):
        for it in range(iter_max[idx]):
            yb = A(theta + b)
            x = (theta + b) + _lambda * (At((y - yb) / (Phi_sum + gamma)))
            theta = _tv_step(x - b, tv_weight, tv_iter_max, multichannel, tvm)
            theta = cnn(theta, nsig, model)
            theta = np.clip(theta, 0, 1)
            b = b - (x - theta)
            if show_iqa and X_orig is not None:
                psnr_all.append(psnr(X_orig, x))
    psnr_, ssim_ = _frame_metrics(X_orig, x)
    return x, psnr_, ssim_, psnr_all


def joint_admmdenoise_cacti(meas, mask, A, At, cnn, projmeth='admm', v0=None, orig=None,
                            iframe=0, nframe=1, MAXB=1., maskdirection='plain', denoiser='tv',
                            iter_max1=50, iter_max2=50, sigma1=None, sigma2=None, **args):
    """``joint_pnp_sci_algo.py:20-59`` with ``gap_joint_denoise`` /
    ``admm_joint_denoise`` (``:81-116``): per block, ``iter_max1`` TV-only
    iterations (sigma1), then ``iter_max2`` TV + CNN iterations (sigma2),
    the second period starting from the first's x."""
    nrow, ncol, nmask = mask.shape
    x_ = np.zeros((nrow, ncol, nmask * nframe), dtype=np.float32)
    psnr_, ssim_, psnrall_ = [], [], []
    begin_time = time.time()
    for kf in range(nframe):
        flip = (maskdirection.lower() == 'updown' and (kf + iframe) % 2 == 1) or \
               (maskdirection.lower() == 'downup' and (kf + iframe) % 2 == 0)
        orig_k = None if orig is None else \
            orig[:, :, (kf + iframe) * nmask:(kf + iframe + 1) * nmask] / MAXB
        meas_k = meas[:, :, kf + iframe] / MAXB
        v0_k = None
        if v0 is not None:
            v0_k = v0[:, :, kf * nmask:(kf + 1) * nmask]
            if flip:
                v0_k = v0_k[:, :, ::-1]
        mask_sum = np.sum(mask, axis=2)
        mask_sum[mask_sum == 0] = 1
        if projmeth.lower() == 'admm':
            x, _, _, _ = joint_admm_denoise(meas_k, mask_sum, A, At, x0=v0_k, X_orig=orig_k,
                                            denoiser='tv', iter_max=iter_max1, sigma=sigma1,
                                            **args)
            x_k, psnr_k, ssim_k, psnrall_k = admm_multistep_denoise(
                meas_k, mask_sum, A, At, cnn, x0=x, X_orig=orig_k, denoiser=denoiser,
                iter_max=iter_max2, sigma=sigma2, **args)
        elif projmeth.lower() == 'gap':
            x, _, _, _ = gap_denoise(meas_k, mask_sum, A, At, x0=v0_k, X_orig=orig_k,
                                     denoiser='tv', iter_max=iter_max1, sigma=sigma1,
                                     **{k: v for k, v in args.items() if k not in ('gamma',)})
            x_k, psnr_k, ssim_k, psnrall_k = gap_multistep_denoise(
                meas_k, mask_sum, A, At, cnn, x0=x, X_orig=orig_k, denoiser=denoiser,
                iter_max=iter_max2, sigma=sigma2, **args)
        else:
            raise ValueError('Unsupported projection method %s' % projmeth.upper())
        if flip:
            x_k = x_k[:, :, ::-1]
            psnr_k = psnr_k[::-1]
            ssim_k = ssim_k[::-1]
            psnrall_k = psnrall_k[::-1]
        t_ = time.time() - begin_time
        x_[:, :, kf * nmask:(kf + 1) * nmask] = x_k
        psnr_.extend(psnr_k)
        ssim_.extend(ssim_k)
        psnrall_.append(psnrall_k)
    return x_, t_, psnr_, ssim_, psnrall_
