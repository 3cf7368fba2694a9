"""CPU oracle: Chambolle total-variation denoiser as the reference path calls it.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, and only as the checker.

The reference path calls scikit-image's ``restoration.denoise_tv_chambolle``
(``PnP_SCI/python/pnp_sci_algo.py:650`` for GAP, ``:812-813`` for ADMM,
``:874`` and ``:895`` for the legacy loops) with ``multichannel=True`` and
the default ``eps``.  scikit-image is a third-party dependency that is not
vendored in the reference; ``PnP_SCI/python/environment.yml:15`` leaves it
unpinned, and the import code (``pnp_sci_algo.py:13-17``: the
``skimage.measure.compare_psnr`` branch and the ``multichannel=`` keyword)
implies scikit-image 0.16.x/0.17.x.  This module restates that release's
published algorithm -- Chambolle (2004), "An Algorithm for Total Variation
Minimization and Applications", J. Math. Imaging Vis. 20:89-97, with
scikit-image's parameters:

* tau = 1 / (2 * ndim); p_0 = 0; gradients are forward differences whose
  last entry along each axis is 0; the divergence is the negative adjoint
  (backward differences with p_{-1} = 0);
* per step k: u_k = f - div p_k (u_0 = f), energy
  E_k = (sum (div p_k)^2 + weight * sum |grad u_k|) / f.size,
  p_{k+1} = (p_k - tau grad u_k) / (1 + tau/weight |grad u_k|);
* stop after step k >= 1 when |E_{k-1} - E_k| < eps * E_0, or when
  k + 1 == n_iter_max; return u_k of the last executed step.

The arithmetic below keeps scikit-image's order of numpy operations, so a
run in float64 is meant to be bit-identical to it.  scikit-image itself is
not installed anywhere this project runs, so that claim is UNPINNED: the
restatement is checked only through the known-answer properties in
``tests/test_oracle.py``: constant frames are fixed points, n_iter_max=1
returns the input, the stop rule, the decrease of Chambolle's dual
objective ||f - div p_k||^2 (the reported energy E_k itself is not
monotone and no test relies on it), and the in-repo MATLAB Chambolle
variant ``PnP_SCI/matlab/algorithms/tvdenoisers/tvdenoise_cham_ITV2D.m:49-93``.
"""
import numpy as np


def _tv_chambolle_nd(image, weight, eps, n_iter_max):
    """One image (any ndim) through the Chambolle iteration.

    Returns ``(out, n_steps, energies)``; ``out`` is the result scikit-image
    returns, ``n_steps`` the number of executed steps and ``energies`` the
    list of E_k values (used by tests for the stop-index check).
    """
    ndim = image.ndim
    p = np.zeros((ndim,) + image.shape, dtype=image.dtype)
    g = np.zeros_like(p)
    d = np.zeros_like(image)
    energies = []
    e_init = e_prev = None
    out = image
    i = 0
    while i < n_iter_max:
        if i > 0:
            # d = -div p: d_j = p_{j-1} - p_j along every axis (p_{-1} = 0)
            d = -p.sum(0)
            for ax in range(ndim):
                dst = [slice(None)] * ndim
                src = [slice(None)] * ndim
                dst[ax] = slice(1, None)
                src[ax] = slice(0, -1)
                d[tuple(dst)] += p[ax][tuple(src)]
            out = image + d
        else:
            out = image
        e = (d ** 2).sum()
        for ax in range(ndim):
            head = [slice(None)] * ndim
            head[ax] = slice(0, -1)
            g[ax][tuple(head)] = np.diff(out, axis=ax)
        norm = np.sqrt((g ** 2).sum(axis=0))[np.newaxis, ...]
        e += weight * norm.sum()
        tau = 1.0 / (2.0 * ndim)
        norm *= tau / weight
        norm += 1.0
        p -= tau * g
        p /= norm
        e /= float(image.size)
        energies.append(e)
        if i == 0:
            e_init = e
            e_prev = e
        else:
            if np.abs(e_prev - e) < eps * e_init:
                break
            e_prev = e
        i += 1
    n_steps = min(i + 1, n_iter_max)
    return out, n_steps, energies


def denoise_tv_chambolle(image, weight=0.1, eps=2.e-4, n_iter_max=200,
                         multichannel=False, threads=1):
    """scikit-image 0.16 ``denoise_tv_chambolle`` semantics (see module doc).

    With ``multichannel=True`` every slice ``image[..., c]`` is denoised as
    an independent image, which is how the GAP/ADMM drivers use it on an
    H x W x B frame stack.  ``threads`` > 1 denoises the slices on a thread
    pool (numpy releases the interpreter lock inside its array loops); the
    slices are independent, so the result is the same.
    """
    image = np.asarray(image)
    if image.dtype.kind != 'f':
        raise TypeError("the oracle TV takes floating-point images only")
    if multichannel:
        out = np.zeros_like(image)

        def one(c):
            out[..., c] = _tv_chambolle_nd(image[..., c], weight, eps, n_iter_max)[0]

        if threads > 1:
            from concurrent.futures import ThreadPoolExecutor
            with ThreadPoolExecutor(max_workers=threads) as ex:
                list(ex.map(one, range(image.shape[-1])))
        else:
            for c in range(image.shape[-1]):
                one(c)
        return out
    return _tv_chambolle_nd(image, weight, eps, n_iter_max)[0]


def tv_chambolle_frames(stack, weight, eps=2.e-4, n_iter_max=200):
    """Per-frame TV of an H x W x B stack with per-frame diagnostics.

    Returns ``(out, steps, energies)`` where ``steps[b]`` is the number of
    executed Chambolle steps of frame b (``n_iter_max`` when no early stop)
    and ``energies[b]`` its list of E_k.
    """
    out = np.zeros_like(stack)
    steps, energies = [], []
    for c in range(stack.shape[-1]):
        u, n, e = _tv_chambolle_nd(stack[..., c], weight, eps, n_iter_max)
        out[..., c] = u
        steps.append(n)
        energies.append(e)
    return out, steps, energies


def tv_cham_itv2d_matlab(f, lam, iters):
    """The in-repo MATLAB Chambolle variant, restated for a cross-check.

    ``PnP_SCI/matlab/algorithms/tvdenoisers/tvdenoise_cham_ITV2D.m:49-93``
    (2-D branch): dt = 1/8, z = div p - lam f, p <- (p + dt grad z) /
    (1 + dt |grad z|), div p with a zero first column/row
    (``il``/``iu`` index the element itself at position 1), no stop test,
    u = f - div p / lam after ``iters`` updates.  With lam = 1/weight and
    p scaled by weight it is the scikit-image recurrence with tau = dt and a
    different first-column divergence; ``tests/test_oracle.py`` uses that
    correspondence.
    """
    f = np.asarray(f, dtype=np.float64)
    dt = 1.0 / 8.0
    p1 = np.zeros_like(f)
    p2 = np.zeros_like(f)
    divp = np.zeros_like(f)
    for _ in range(iters):
        z = divp - f * lam
        z1 = np.zeros_like(z)
        z2 = np.zeros_like(z)
        z1[:, :-1] = z[:, 1:] - z[:, :-1]
        z2[:-1, :] = z[1:, :] - z[:-1, :]
        denom = 1.0 + dt * np.sqrt(z1 ** 2 + z2 ** 2)
        p1 = (p1 + dt * z1) / denom
        p2 = (p2 + dt * z2) / denom
        divp = np.zeros_like(f)
        divp[:, 1:] = p1[:, 1:] - p1[:, :-1]
        divp[1:, :] += p2[1:, :] - p2[:-1, :]
    return f - divp / lam
