"""CPU restatement of the MATLAB TV denoisers of PnP_SCI (test infrastructure).

These are the denoisers that the MATLAB twin of the GAP loop selects with its
``tvm`` switch (PnP_SCI/matlab/algorithms/gapdenoise.m:92-112).  Each
function restates one file of PnP_SCI/matlab/algorithms/tvdenoisers/ in
float64 numpy on an H x W x B stack (MATLAB's frames-last layout), with
MATLAB's own single-frame behaviour: MATLAB sees an H x W x 1 array as 2-D,
and several of these files take a different branch for it.

Parity status: unpinned against MATLAB (neither MATLAB nor Octave is
available, and the reference ships no outputs of these files).  The
restatements are checked against each other where the files coincide
(tests/test_oracle_tv_matlab.py).

Only tests/, the smoke check and the bench's CPU leg import this module.
"""
import numpy as np

# gapdenoise.m:92-112 -- the tvm names, the denoiser each one calls, and how
# it maps (tvweight) to the denoiser's parameter and iteration count
TVM = {
    "ATV_ClipA": ("clip_a", lambda w: w, 5),
    "ATV_ClipB": ("clip_b", lambda w: w, 5),
    "ATV_cham": ("cham_atv", lambda w: 1.0 / w, 5),
    "ATV_FGP": ("fgp_atv", lambda w: w, 2),
    "ITV2D_cham": ("cham_itv2d", lambda w: 1.0 / w, 5),
    "ITV2D_FGP": ("fgp_itv2d", lambda w: w, 2),
    "ITV3D_cham": ("cham_itv3d", lambda w: 1.0 / w, 5),
    "ITV3D_FGP": ("fgp_itv3d", lambda w: w, 2),
}


def _stack(f):
    f = np.asarray(f, np.float64)
    if f.ndim == 2:
        f = f[:, :, None]
    assert f.ndim == 3 and f.shape[0] >= 2 and f.shape[1] >= 2, "H, W >= 2"
    return f


# ------------------------------------------------------------ clip family
# TV_denoising.m:59-84 and TV_denoising_clip_LB.m:60-85 (same helpers)
def _dh(x):  # diff(x,1,2)
    return x[:, 1:] - x[:, :-1]


def _dv(x):  # diff(x)
    return x[1:] - x[:-1]


def _dht(z):  # [-x(:,1) -diff(x,1,2) x(:,end)]
    return np.concatenate([-z[:, :1], -(z[:, 1:] - z[:, :-1]), z[:, -1:]], axis=1)


def _dvt(z):  # [-x(1,:); -diff(x); x(end,:)]
    return np.concatenate([-z[:1], -(z[1:] - z[:-1]), z[-1:]], axis=0)


def _clip(x, lam):  # sign(x).*(min(abs(x),lambda))
    return np.sign(x) * np.minimum(np.abs(x), lam)


def tv_denoising(y0, lam, iters=100):
    """ATV_ClipA: TV_denoising.m:1-58 (alpha = 5).  Per iteration
    x0 = ((y0 - dht(zh)) + (y0 - dvt(zv))) / 2, then both duals take a
    clipped step of 1/alpha along the forward differences of x0 (clip at
    lambda/2).  Returns x0 of the last iteration."""
    y0 = _stack(y0)
    H, W, B = y0.shape
    alpha = 5.0
    zh = np.zeros((H, W - 1, B))
    zv = np.zeros((H - 1, W, B))
    x0 = None
    for _ in range(iters):
        x0h = y0 - _dht(zh)
        x0v = y0 - _dvt(zv)
        x0 = (x0h + x0v) / 2
        zh = _clip(zh + 1 / alpha * _dh(x0), lam / 2)
        zv = _clip(zv + 1 / alpha * _dv(x0), lam / 2)
    return x0


def tv_denoising_clip_lb(y0, lam, iters=20):
    """ATV_ClipB: TV_denoising_clip_LB.m:1-58.  For a stack of more than
    one frame (the 3-D branch, :23-34): x0 = y0 - dht(zh) - dvt(zv) and
    the duals are clipped at lambda.  A single frame takes the 2-D branch
    (:12-22), which is TV_denoising's update."""
    y0 = _stack(y0)
    if y0.shape[2] == 1:
        return tv_denoising(y0, lam, iters)
    H, W, B = y0.shape
    alpha = 5.0
    zh = np.zeros((H, W - 1, B))
    zv = np.zeros((H - 1, W, B))
    x0 = None
    for _ in range(iters):
        x0 = y0 - _dht(zh) - _dvt(zv)
        zh = _clip(zh + 1 / alpha * _dh(x0), lam)
        zv = _clip(zv + 1 / alpha * _dv(x0), lam)
    return x0


# -------------------------------------------------------- Chambolle family
def _cham(f, lam, iters, dt, mode):
    """Common body of tvdenoise_cham_{ITV2D,ATV2D,ITV3D}.m:49-93 (Pascal
    Getreuer's Chambolle iteration): z = divp - lambda f; z1, z2 forward
    differences with a replicated last column / row (0 there); dual update
    per `mode`; divp = p1 - p1(:,il) + p2 - p2(iu,:) with il, iu repeating
    the first column / row (so divp takes no p at column / row 1);
    u = f - divp / lambda."""
    f = _stack(f)
    if lam < 0:
        raise ValueError("Parameter lambda must be nonnegative.")
    H, W, B = f.shape
    ir = np.r_[1:W, W - 1]
    idn = np.r_[1:H, H - 1]
    il = np.r_[0, 0:W - 1]
    iu = np.r_[0, 0:H - 1]
    p1 = np.zeros_like(f)
    p2 = np.zeros_like(f)
    divp = np.zeros_like(f)
    for _ in range(iters):
        z = divp - f * lam
        z1 = z[:, ir] - z
        z2 = z[idn, :] - z
        if mode == "iso":
            denom = 1 + dt * np.sqrt(z1 ** 2 + z2 ** 2)
            p1 = (p1 + dt * z1) / denom
            p2 = (p2 + dt * z2) / denom
        elif mode == "iso_coupled":
            denom = 1 + dt * np.sqrt(np.sum(z1 ** 2 + z2 ** 2, axis=2, keepdims=True))
            p1 = (p1 + dt * z1) / denom
            p2 = (p2 + dt * z2) / denom
        else:  # "aniso"
            p1 = (p1 + dt * z1) / np.maximum(1, np.abs(p1 + dt * z1))
            p2 = (p2 + dt * z2) / np.maximum(1, np.abs(p2 + dt * z2))
        divp = p1 - p1[:, il] + p2 - p2[iu, :]
    return f - divp / lam


def tvdenoise_cham_itv2d(f, lam, iters):
    """ITV2D_cham: tvdenoise_cham_ITV2D.m:49-94, dt = 1/8, per-frame
    isotropic norm (both branches, :62-73 and :74-91)."""
    return _cham(f, lam, iters, 1 / 8, "iso")


def tvdenoise_cham_atv2d(f, lam, iters):
    """ATV_cham: tvdenoise_cham_ATV2D.m:48-91, dt = 1/8.  A stack of more
    than one frame (:72-88) projects each dual component on [-1, 1]
    (anisotropic); a single frame takes the isotropic 2-D branch (:60-71)."""
    f = _stack(f)
    return _cham(f, lam, iters, 1 / 8, "iso" if f.shape[2] == 1 else "aniso")


def tvdenoise_cham_itv3d(f, lam, iters):
    """ITV3D_cham: tvdenoise_cham_ITV3D.m:49-94, dt = 1/4, the norm of the
    gradient summed over all frames of a pixel (:83-84); one frame gives
    the per-frame norm."""
    return _cham(f, lam, iters, 1 / 4, "iso_coupled")


# ------------------------------------------------------------ FGP family
def _lforward(P1, P2):
    """Lforward_3d (fgp_denoise_ITV2D.m:135-159)."""
    m, n, B = P1.shape[0] + 1, P1.shape[1], P1.shape[2]
    X = np.zeros((m, n, B))
    X[: m - 1] = P1
    X[:, : n - 1] = X[:, : n - 1] + P2
    X[1:m] = X[1:m] - P1
    X[:, 1:n] = X[:, 1:n] - P2
    return X


def _ltrans(X):
    """Ltrans_3d (fgp_denoise_ITV2D.m:162-168)."""
    return X[:-1] - X[1:], X[:, :-1] - X[:, 1:]


def _fgp(Xobs, lam, maxiter, mode):
    """Common body of fgp_denoise_{ITV2D,ATV2D,ITV3D}.m:51-131 (Beck and
    Teboulle's fast gradient projection on the dual).  The stopping counter
    is never incremented (its update is commented out, :113-118), so the
    loop runs maxiter times.  Returns D of the last iteration."""
    Xobs = _stack(Xobs)
    m, n, B = Xobs.shape
    P1 = np.zeros((m - 1, n, B))
    P2 = np.zeros((m, n - 1, B))
    R1 = np.zeros((m - 1, n, B))
    R2 = np.zeros((m, n - 1, B))
    tkp1 = 1.0
    D = np.zeros((m, n, B))
    for _ in range(maxiter):
        Pold1, Pold2 = P1, P2
        tk = tkp1
        D = Xobs - lam * _lforward(R1, R2)
        Q1, Q2 = _ltrans(D)
        P1 = R1 + 1 / (8 * lam) * Q1
        P2 = R2 + 1 / (8 * lam) * Q2
        if mode == "aniso":
            P1 = P1 / np.maximum(np.abs(P1), 1)
            P2 = P2 / np.maximum(np.abs(P2), 1)
        else:
            A = (np.concatenate([P1, np.zeros((1, n, B))], axis=0) ** 2 +
                 np.concatenate([P2, np.zeros((m, 1, B))], axis=1) ** 2)
            if mode == "iso":
                A = np.sqrt(np.maximum(A, 1))
            else:  # "iso_coupled"
                A = np.repeat(np.sqrt(np.maximum(np.sum(A, axis=2, keepdims=True), 1)), B,
                              axis=2)
            P1 = P1 / A[: m - 1]
            P2 = P2 / A[:, : n - 1]
        tkp1 = (1 + np.sqrt(1 + 4 * tk ** 2)) / 2
        R1 = P1 + (tk - 1) / tkp1 * (P1 - Pold1)
        R2 = P2 + (tk - 1) / tkp1 * (P2 - Pold2)
    return D


def fgp_denoise_itv2d(Xobs, lam, maxiter):
    """ITV2D_FGP: fgp_denoise_ITV2D.m:1-133, isotropic per frame (:97-100)."""
    return _fgp(Xobs, lam, maxiter, "iso")


def fgp_denoise_atv2d(Xobs, lam, maxiter):
    """ATV_FGP: fgp_denoise_ATV2D.m:1-133, each component on [-1, 1]
    (:102-103)."""
    return _fgp(Xobs, lam, maxiter, "aniso")


def fgp_denoise_itv3d(Xobs, lam, maxiter):
    """ITV3D_FGP: fgp_denoise_ITV3D.m:1-134, the norm summed over frames
    (:98-99)."""
    return _fgp(Xobs, lam, maxiter, "iso_coupled")


_FN = {
    "clip_a": tv_denoising,
    "clip_b": tv_denoising_clip_lb,
    "cham_atv": tvdenoise_cham_atv2d,
    "cham_itv2d": tvdenoise_cham_itv2d,
    "cham_itv3d": tvdenoise_cham_itv3d,
    "fgp_atv": fgp_denoise_atv2d,
    "fgp_itv2d": fgp_denoise_itv2d,
    "fgp_itv3d": fgp_denoise_itv3d,
}


def tv_by_name(v, tvm, tvweight):
    """The denoising step of gapdenoise.m:92-112 for `tvm`, on H x W x B."""
    kind, param, iters = TVM[tvm]
    return _FN[kind](v, param(tvweight), iters)


def gap_tv_matlab(y, mask, tvm, tvweight, iters, lam=1.0, acc=True, v0=None):
    """The GAP loop of gapdenoise.m:70-92 with a TV denoiser from the tvm
    switch (float64): yb = A(v); acc: y1 += y - yb, v += lambda At((y1 -
    yb) / Phisum); else v += lambda At((y - yb) / Phisum); v = TV(v)."""
    mask = np.asarray(mask, np.float64)
    y = np.asarray(y, np.float64)
    phisum = mask.sum(axis=2)
    phisum[phisum == 0] = 1
    v = (mask * y[:, :, None]).copy() if v0 is None else np.array(v0, np.float64)
    y1 = np.zeros_like(y)
    for _ in range(iters):
        yb = np.sum(v * mask, axis=2)
        if acc:
            y1 = y1 + (y - yb)
            v = v + lam * (mask * ((y1 - yb) / phisum)[:, :, None])
        else:
            v = v + lam * (mask * ((y - yb) / phisum)[:, :, None])
        v = tv_by_name(v, tvm, tvweight)
    return v
