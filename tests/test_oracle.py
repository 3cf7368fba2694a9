"""The oracle pinned against the reference's own outputs (no GPU needed).

Fixtures come from ``tests/golden/make_golden.py``, which ran the
reference's ``utils.py`` / ``pnp_sci_algo.py`` themselves.  The numpy port
must reproduce them bit for bit; the C oracle must agree with the numpy
port to 1e-12 relative.  The third-party TV restatement is checked through
known-answer properties (its parity with scikit-image is unpinned).
"""
import json

import numpy as np
import pytest

from oracle import reference_port as port
from oracle import c_oracle
from oracle.tv_chambolle import (denoise_tv_chambolle, tv_chambolle_frames,
                                 tv_cham_itv2d_matlab, _tv_chambolle_nd)
import sci_algorithms_gb300.datasets as ds


def _cacti_args(g):
    return json.loads(str(g["args_json"]))


def _run_port_cacti(g):
    mask, meas, orig = g["mask"], g["meas"], g["orig"]
    A = lambda x: port.A_(x, mask)  # noqa: E731
    At = lambda y: port.At_(y, mask)  # noqa: E731
    v0 = g["v0"] if "v0" in g else None
    return port.admmdenoise_cacti(
        meas, mask, A, At, projmeth=str(g["projmeth"]), v0=v0, orig=orig,
        iframe=int(g["iframe"]), nframe=int(g["nframe"]), MAXB=float(g["MAXB"]),
        maskdirection=str(g["maskdirection"]), **_cacti_args(g))


def test_ops_bit_exact(golden):
    g = golden("ops")
    assert np.array_equal(port.A_(g["x"], g["phi"]), g["A"])
    assert np.array_equal(port.At_(g["y"], g["phi"]), g["At"])
    assert port.psnr(g["x"], g["x"] + 0.01 * g["y"][..., None]) == g["psnr"]
    assert port.psnr(g["x"], g["x"]) == 100 == g["psnr_equal"]


@pytest.mark.parametrize("case", ["gap_acc", "gap_plain", "gap_tv30", "admm",
                                  "gap_updown", "admm_downup"])
def test_driver_bit_exact(golden, case):
    g = golden(case)
    x_, _t, psnr_, ssim_, psnrall_ = _run_port_cacti(g)
    assert np.array_equal(x_.astype(np.float64), g["x"])
    assert np.array_equal(np.array(psnr_), g["psnr"])
    assert np.array_equal(np.array(ssim_), g["ssim"])
    assert np.array_equal(np.array(psnrall_), g["psnrall"])


def test_legacy_loops_bit_exact(golden):
    g = golden("legacy")
    msum = np.sum(g["mask"], axis=2)
    msum[msum == 0] = 1
    v = port.ADMM_TV_rec(g["meas"], g["mask"], port.A_, port.At_, msum, 6, 1.0,
                         0.1, 20, 20, 4, 0.01, g["orig"])
    f = port.GAP_TV_rec(g["meas"], g["mask"], port.A_, port.At_, msum, 5, 1.0,
                        0.1, 20, 20, 4, g["orig"])
    assert np.array_equal(v, g["admm"])
    assert np.array_equal(f, g["gap"])


@pytest.mark.parametrize("case", ["bayer_gap", "bayer_gap_acc"])
def test_bayer_gap_bit_exact(golden, case):
    g = golden(case)
    x, psnr_, ssim_, psnrall_ = port.gap_denoise_bayer(
        g["meas"], g["mask"], _lambda=1, accelerate=bool(g["accelerate"]), iter_max=8,
        tv_weight=0.1, tv_iter_max=5, X_orig=g["orig"])
    assert np.array_equal(np.asarray(x, np.float64), g["x"])
    assert np.array_equal(np.array(psnr_), g["psnr"])
    assert np.array_equal(np.array(ssim_), g["ssim"])
    assert np.array_equal(np.array(psnrall_), g["psnrall"])


def test_bayer_admm_is_four_channel_admm(golden):
    """The ADMM Bayer restatement (the reference's raises at :400) is the
    per-channel admm_denoise on the four sub-lattices."""
    g = golden("bayer_gap")
    y, mask = g["meas"], g["mask"]
    x, psnr_all = port.admm_denoise_bayer(y, mask, gamma=0.02, iter_max=6, tv_weight=0.1,
                                          X_orig=g["orig"])
    assert len(psnr_all) == 6
    for b0, b1 in port.BAYER:
        m = mask[b0::2, b1::2].astype(np.float32)
        yc = y[b0::2, b1::2].astype(np.float32)
        ms = m.sum(axis=2)
        ms[ms == 0] = 1
        xc, _, _, _ = port.admm_denoise(yc, ms, lambda v: port.A_(v, m),
                                        lambda r: port.At_(r, m), gamma=0.02, iter_max=6,
                                        tv_weight=0.1)
        assert np.allclose(x[b0::2, b1::2], xc, rtol=0, atol=1e-5)


@pytest.mark.parametrize("case", ["joint_gap", "joint_admm"])
def test_joint_tv_cnn_loops_bit_exact(golden, case):
    """joint_admmdenoise_cacti (joint_pnp_sci_algo.py) with the box-blur
    stand-in CNN, against the reference's own run."""
    g = golden(case)
    mask = g["mask"]
    args = json.loads(str(g["args_json"]))
    x_, _t, psnr_, ssim_, psnrall_ = port.joint_admmdenoise_cacti(
        g["meas"], mask, lambda x: port.A_(x, mask), lambda y: port.At_(y, mask),
        port.cnn_stand_in, projmeth=case.split("_")[1], orig=g["orig"],
        denoiser=str(g["denoiser"]), **args)
    assert np.array_equal(x_.astype(np.float64), g["x"])
    assert np.array_equal(np.array(psnr_), g["psnr"])
    assert np.array_equal(np.array(ssim_), g["ssim"])
    assert np.array_equal(np.array(psnrall_), g["psnrall"])


def test_config0_inputs_and_digest(golden):
    import hashlib
    g = golden("config0")
    orig, mask, meas = ds.config0()

    def dg(a):
        return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()
    assert dg(orig) == str(g["orig_digest"])
    assert dg(mask) == str(g["mask_digest"])
    assert dg(meas) == str(g["meas_digest"])


# ------------------------------------------------------------ TV properties
def test_tv_constant_frame_unchanged():
    f = np.full((17, 23, 3), 0.37)
    u = denoise_tv_chambolle(f, 0.2, n_iter_max=7, multichannel=True)
    assert np.array_equal(u, f)


def test_tv_single_step_is_identity():
    rng = np.random.default_rng(3)
    f = rng.random((19, 11, 2))
    assert np.array_equal(denoise_tv_chambolle(f, 0.3, n_iter_max=1, multichannel=True), f)


def test_tv_stop_rule():
    rng = np.random.default_rng(4)
    f = rng.random((40, 33))
    _, n, e = _tv_chambolle_nd(f, 0.1, 2e-4, 400)
    assert n < 400  # the stop test fires
    assert len(e) == n
    # (E_k is scikit-image's stopping heuristic, not a monotone objective:
    # it dips after the first step and then rises towards its limit.)
    # stop at the first k with |E_{k-1}-E_k| < eps E_0
    k_stop = next(k for k in range(1, len(e)) if abs(e[k - 1] - e[k]) < 2e-4 * e[0])
    assert n == k_stop + 1


def test_tv_matches_matlab_variant_in_the_interior():
    """Same ROF problem as tvdenoise_cham_ITV2D.m with lambda = 1/weight:
    after convergence both agree away from the first row/column (where the
    MATLAB divergence differs)."""
    rng = np.random.default_rng(5)
    f = np.cumsum(np.cumsum(rng.standard_normal((28, 28)), 0), 1)
    f = (f - f.min()) / (f.max() - f.min())
    w = 0.08
    u_sk = _tv_chambolle_nd(f, w, 0.0, 3000)[0]
    u_ml = tv_cham_itv2d_matlab(f, 1.0 / w, 6000)
    inner = (slice(10, None), slice(10, None))
    assert np.max(np.abs(u_sk[inner] - u_ml[inner])) < 1e-5
    # ... and the first-row/column divergence is where they differ
    assert np.max(np.abs(u_sk[:2] - u_ml[:2])) > 1e-4


def test_tv_frames_diagnostics_match_wrapper():
    rng = np.random.default_rng(6)
    f = rng.random((15, 14, 4))
    u1 = denoise_tv_chambolle(f, 0.15, n_iter_max=60, multichannel=True)
    u2, steps, _ = tv_chambolle_frames(f, 0.15, n_iter_max=60)
    assert np.array_equal(u1, u2)
    assert all(1 <= s <= 60 for s in steps)


# ---------------------------------------------------------------- C oracle
def test_c_oracle_tv_matches_port():
    rng = np.random.default_rng(8)
    f = rng.random((21, 18, 5))
    for n_iter in (1, 2, 5, 40):
        ref, steps, _ = tv_chambolle_frames(f, 0.12, n_iter_max=n_iter)
        u, csteps, _ = c_oracle.tv_chambolle(c_oracle.planar(f), 0.12, n_iter)
        assert list(csteps) == steps
        np.testing.assert_allclose(c_oracle.unplanar(u), ref, rtol=0, atol=1e-13)


@pytest.mark.parametrize("case", ["gap_acc", "gap_plain", "admm"])
def test_c_oracle_solver_matches_golden(golden, case):
    g = golden(case)
    args = _cacti_args(g)
    mask, meas, orig = g["mask"], g["meas"][..., 0], g["orig"]
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    iters = args["iter_max"]
    iters = sum(iters) if isinstance(iters, list) else iters
    x0 = c_oracle.planar(port.At_(meas, mask))
    if str(g["projmeth"]) == "gap":
        x, pa = c_oracle.gap_tv(meas, c_oracle.planar(mask), msum, x0, iters,
                                lambdas=args["_lambda"], weights=args["tv_weight"],
                                tv_iter_max=args["tv_iter_max"],
                                accelerate=args["accelerate"],
                                orig_bhw=c_oracle.planar(orig))
    else:
        x, pa = c_oracle.admm_tv(meas, c_oracle.planar(mask), msum, x0, iters,
                                 lambdas=args["_lambda"], weights=args["tv_weight"],
                                 gamma=args["gamma"], tv_iter_max=args["tv_iter_max"],
                                 orig_bhw=c_oracle.planar(orig))
    ref = g["x"]
    rel = np.linalg.norm(c_oracle.unplanar(x) - ref) / np.linalg.norm(ref)
    # x_ of the driver is stored as float32 (pnp_sci_algo.py:494)
    assert rel < 1e-7
    np.testing.assert_allclose(pa, g["psnrall"][0], rtol=1e-6)


def test_gap_step_with_unit_mask_and_one_frame_returns_y():
    """Known answer: with Phi = 1 and B = 1, A x = x and Phi_sum = 1, so one
    GAP projection (lambda = 1, pnp_sci_algo.py:645) maps any x to y."""
    rng = np.random.default_rng(3)
    mask = np.ones((20, 24, 1))
    x = rng.random((20, 24, 1))
    y = rng.random((20, 24))
    msum = mask.sum(axis=2)
    x1 = x + 1.0 * port.At_((y - port.A_(x, mask)) / msum, mask)
    np.testing.assert_allclose(x1[..., 0], y, rtol=0, atol=1e-15)


def test_tv_dual_objective_is_non_increasing():
    """Chambolle's iteration decreases its dual objective ||f - div p_k||^2
    = ||u_k||^2 step by step (Chambolle 2004, for the step 1/4 scikit-image
    uses as well, checked here), while scikit-image's reported energy
    E_k = (||f - u_k||^2 + w TV(u_k)) / (H W) need not decrease (its stop
    rule compares successive values only)."""
    rng = np.random.default_rng(4)
    f = np.concatenate([rng.random((1, 40, 50)),
                        np.cumsum(rng.standard_normal((1, 40, 50)), axis=2) * 0.05])
    rises = 0
    for w in (0.02, 0.1, 0.5):
        norms = []
        for K in range(1, 16):
            u, steps, en = c_oracle.tv_chambolle(f, w, K, eps=0.0)
            norms.append((u ** 2).sum(axis=(1, 2)))
        d = np.diff(np.array(norms), axis=0)
        assert np.all(d <= 1e-12 * norms[0]), w
        e = c_oracle.tv_chambolle(f, w, 15, eps=0.0)[2]
        rises += int((np.diff(e, axis=1) > 0).sum())
    assert rises > 0  # the reported energy is not monotone: no test may assume it
