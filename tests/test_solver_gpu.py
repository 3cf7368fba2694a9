"""GPU GAP-TV / ADMM-TV drivers against the reference's own outputs.

The fixtures were produced by the reference's ``admmdenoise_cacti`` /
``gap_denoise`` / ``admm_denoise`` / ``ADMM_TV_rec`` (float64 numpy, see
``tests/golden/make_golden.py``).  The GPU computes in float32; the bar is
the benchmark spec's tolerance, relative L2 <= 1e-4 to the float64 result, and
per-iteration PSNR within 0.01 dB.
"""
import json

import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev
from oracle import reference_port as port

pytestmark = pytest.mark.gpu

REL_L2 = 1e-4
PSNR_TOL = 1e-2


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run_case(g, A=None, At=None, **extra):
    mask = g["mask"]
    if A is None:
        A, At = sci.make_ops(mask)
    args = json.loads(str(g["args_json"]))
    args.update(extra)
    v0 = g["v0"] if "v0" in g else None
    return sci.admmdenoise_cacti(g["meas"], mask, A, At, projmeth=str(g["projmeth"]), v0=v0,
                                 orig=g["orig"], iframe=int(g["iframe"]),
                                 nframe=int(g["nframe"]), MAXB=float(g["MAXB"]),
                                 maskdirection=str(g["maskdirection"]), **args)


@pytest.mark.parametrize("case", ["gap_acc", "gap_plain", "gap_tv30", "admm", "gap_updown",
                                  "admm_downup"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_cacti_matches_reference(golden, case, use_graph):
    g = golden(case)
    x_, t_, psnr_, ssim_, psnrall_ = run_case(g, use_graph=use_graph)
    assert x_.dtype == np.float32 and x_.shape == g["x"].shape
    assert rel(x_, g["x"]) < REL_L2
    assert np.max(np.abs(np.array(psnr_) - g["psnr"])) < PSNR_TOL
    assert np.max(np.abs(np.array(ssim_) - g["ssim"])) < 1e-4
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < PSNR_TOL
    assert t_ >= 0


def test_plugin_path_with_reference_style_closures(golden):
    """A = lambda x: A_(x, mask) with the package's A_ (foreign callables)."""
    g = golden("gap_acc")
    mask = g["mask"]
    A = lambda x: sci.A_(x, mask)  # noqa: E731  (pnp_sci_test_orig.py:147)
    At = lambda y: sci.At_(y, mask)  # noqa: E731
    x_, _, psnr_, _, _ = run_case(g, A, At)
    assert rel(x_, g["x"]) < REL_L2
    g = golden("admm")
    mask = g["mask"]
    x_, _, _, _, psnrall_ = run_case(g, lambda x: sci.A_(x, mask), lambda y: sci.At_(y, mask))
    assert rel(x_, g["x"]) < REL_L2
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < PSNR_TOL


def test_config0_against_reference(golden):
    """256 x 256 x 8, 40 GAP-acc iterations, x0 = At(y / Phi_sum)."""
    g = golden("config0")
    orig, mask, meas = sci.datasets.config0()
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    v0 = port.At_(meas / msum, mask)
    A, At = sci.make_ops(mask)
    x, psnr_, ssim_, psnr_all = sci.gap_denoise(meas, msum, A, At, _lambda=1, accelerate=True,
                                                iter_max=40, tv_weight=0.1, tv_iter_max=5,
                                                x0=v0, X_orig=orig)
    r = rel(x, g["x_f32"])
    dpsnr = np.mean(psnr_) - np.mean(g["psnr"])
    print("config0: rel L2 %.3e, dPSNR %.4f dB" % (r, dpsnr))
    assert r < REL_L2
    assert abs(dpsnr) < PSNR_TOL
    assert np.max(np.abs(np.array(psnr_all) - g["psnrall"])) < PSNR_TOL


def test_legacy_loops(golden):
    g = golden("legacy")
    msum = g["mask"].sum(axis=2)
    msum[msum == 0] = 1
    v = sci.ADMM_TV_rec(g["meas"], g["mask"], sci.A_, sci.At_, msum, 6, 1.0, 0.1, 20, 20, 4,
                        0.01, g["orig"])
    f = sci.GAP_TV_rec(g["meas"], g["mask"], sci.A_, sci.At_, msum, 5, 1.0, 0.1, 20, 20, 4,
                       g["orig"])
    assert rel(v, g["admm"]) < REL_L2
    assert rel(f, g["gap"]) < REL_L2


def test_torch_inputs_stay_on_device(golden):
    g = golden("gap_acc")
    dev = _dev.device()
    meas = torch.from_numpy(g["meas"]).to(dev)
    mask = torch.from_numpy(g["mask"]).to(dev)
    A, At = sci.make_ops(mask)
    args = json.loads(str(g["args_json"]))
    x_, _, _, _, _ = sci.admmdenoise_cacti(meas, mask, A, At, projmeth="gap", **args)
    assert x_.is_cuda and x_.dtype == torch.float32
    assert rel(x_.cpu().numpy(), g["x"]) < REL_L2


def test_annealed_schedule_matches_oracle():
    """Per-iteration tv_weight / lambda schedules (the 0.2 -> 0.05 annealing)."""
    orig, mask, meas = sci.datasets.video_config(64, 72, 8, noise_rel=0.01)
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    w = port.annealed_weights(0.2, 0.05, 15)
    lam = np.linspace(1.0, 0.8, 15)
    Ar = lambda x: port.A_(x, mask)  # noqa: E731
    Atr = lambda y: port.At_(y, mask)  # noqa: E731
    A, At = sci.make_ops(mask)
    for fn, rfn, kw in ((sci.gap_denoise, port.gap_denoise, {}),
                        (sci.admm_denoise, port.admm_denoise, {"gamma": 0.01})):
        ref = rfn(meas, msum, Ar, Atr, _lambda=lam, iter_max=15, tv_weight=w, tv_iter_max=5,
                  X_orig=orig, **kw)
        out = fn(meas, msum, A, At, _lambda=lam, iter_max=15, tv_weight=w, tv_iter_max=5,
                 X_orig=orig, **kw)
        assert rel(out[0], ref[0]) < REL_L2
        assert np.max(np.abs(np.array(out[3]) - ref[3])) < PSNR_TOL


def test_graph_replay_is_bitwise_stable():
    orig, mask, meas = sci.datasets.video_config(48, 64, 8)
    op = sci.MaskOperator(mask)
    s = sci.Solver(op, "gap", 8, 1.0, 0.1, 5, use_graph=True)
    y = _dev.plane(meas)
    a = s.run(y).clone()
    b = s.run(y).clone()
    s2 = sci.Solver(op, "gap", 8, 1.0, 0.1, 5, use_graph=False)
    c = s2.run(y).clone()
    assert torch.equal(a, b) and torch.equal(a, c)


def test_float_mask_and_packed_mask_agree(monkeypatch):
    """The ADMM projection kernels on a float mask and on the packed mask
    give the same bits (the packed mask's default fused iteration is
    checked against this loop in test_fused_admm_iteration)."""
    monkeypatch.setenv("SCI_ADMM_FUSED", "0")
    orig, mask, meas = sci.datasets.video_config(40, 56, 8)
    op = sci.MaskOperator(mask)
    y = _dev.plane(meas)
    a = sci.Solver(op, "admm", 6, 1.0, 0.1, 5, use_bits=True).run(y).clone()
    b = sci.Solver(op, "admm", 6, 1.0, 0.1, 5, use_bits=False).run(y).clone()
    assert torch.equal(a, b)


def test_run_host_end_to_end():
    orig, mask, meas = sci.datasets.video_config(32, 40, 8)
    op = sci.MaskOperator(mask)
    s = sci.Solver(op, "gap", 5, 1.0, 0.1, 5)
    y_host = torch.from_numpy(meas.astype(np.float32)).pin_memory()
    x_host = s.run_host(y_host)
    assert not x_host.is_cuda
    ref = s.run(_dev.plane(meas)).cpu()
    assert torch.equal(x_host, ref)


@pytest.mark.parametrize("tvm", ["tv_chambolle", "ATV_ClipA", "ITV3D_cham"])
@pytest.mark.parametrize("with_orig", [False, True])
def test_admm_multiplier_from_tv_input_is_bitwise_equal(monkeypatch, tvm, with_orig):
    """ADMM forming b = theta - v in the projection (no residual written by
    the TV) against the stored-residual loop (SCI_ADMM_B_FROM_V=0)."""
    monkeypatch.setenv("SCI_ADMM_FUSED", "0")
    orig, mask, meas = sci.datasets.video_config(64, 96, 8, noise_rel=0.01)
    op = sci.MaskOperator(mask)
    y = _dev.plane(meas)
    o = _dev.planar(orig) if with_orig else None
    gam = np.linspace(0.01, 0.02, 7).astype(np.float32)
    a = sci.Solver(op, "admm", 7, 1.0, 0.1, 5, gammas=gam, tvm=tvm)
    xa = a.run(y, orig=o).clone()
    monkeypatch.setenv("SCI_ADMM_B_FROM_V", "0")
    b = sci.Solver(op, "admm", 7, 1.0, 0.1, 5, gammas=gam, tvm=tvm)
    xb = b.run(y, orig=o).clone()
    assert torch.equal(xa, xb)
    if with_orig:  # the float64 atomic sums of the squared error may differ in order
        assert np.allclose(a.psnr_all(), b.psnr_all(), rtol=0, atol=1e-9)


def test_run_host_many_pipelined():
    """Several measurements through the pipelined host API: each result
    equals its own device solve (the alternating slots and the copy stream
    never hand back a slot's result before its copy-out ends)."""
    H, W, B = 48, 64, 8
    op = None
    ys, refs = [], []
    for k in range(5):
        _, mask, meas = sci.datasets.video_config(H, W, B, seeds=(k, 100, 200 + k))
        if op is None:
            op = sci.MaskOperator(mask)
        ys.append(torch.from_numpy(meas.astype(np.float32)).pin_memory())
    s = sci.Solver(op, "gap", 6, 1.0, 0.1, 5)
    for y in ys:
        refs.append(s.run(y.cuda()).cpu().clone())
    xs = [torch.empty((B, H, W), dtype=torch.float32).pin_memory() for _ in ys]
    s.run_host_many(ys, xs)
    for x, r in zip(xs, refs):
        assert torch.equal(x, r)
    with pytest.raises(ValueError):
        s.run_host_many(ys, xs[:2])


@pytest.mark.parametrize("eps", [2e-4, 0.05])
@pytest.mark.parametrize("iters", [7, 8])
@pytest.mark.parametrize("shape,cpl", [((64, 96, 8), None), ((40, 1040, 6), None),
                                       ((70, 520, 12), "2"), ((33, 1032, 5), "4"),
                                       ((64, 96, 8), "4")])
def test_fused_projection_path_is_bitwise_equal(monkeypatch, eps, iters, shape, cpl):
    """The fused iteration (residual map + projection applied while the TV
    kernel loads x) against the two-kernel iteration, including early stops
    of the TV inside the fused kernel (eps = 0.05), on 2 and 4 columns per
    lane of the lean TV pass."""
    if cpl is not None:
        monkeypatch.setenv("SCI_TV_CPL", cpl)
    orig, mask, meas = sci.datasets.video_config(*shape)
    op = sci.MaskOperator(mask)
    y = _dev.plane(meas)
    monkeypatch.setenv("SCI_FUSED_PROJ", "1")
    fused = sci.Solver(op, "gap", iters, 1.0, 0.1, 5, eps=eps, use_graph=False)
    a = fused.run(y, tv_steps=True).clone()
    sa = fused.tv_steps.clone()
    monkeypatch.setenv("SCI_FUSED_PROJ", "0")
    plain = sci.Solver(op, "gap", iters, 1.0, 0.1, 5, eps=eps, use_graph=False)
    b = plain.run(y, tv_steps=True).clone()
    assert torch.equal(a, b)
    assert torch.equal(sa, plain.tv_steps)
    if eps > 0.01:
        assert int((sa < 5).sum()) > 0  # the stop test fired somewhere


@pytest.mark.parametrize("kind,acc,bits,fused", [
    ("gap", True, True, False), ("gap", False, True, False), ("gap", True, False, False),
    ("gap", True, True, True), ("gap", False, True, True), ("admm", True, True, False),
    ("admm", True, False, False), ("admm", True, True, True)])
def test_projection_residual_norm_matches_oracle(monkeypatch, kind, acc, bits, fused):
    """The FP64 ||r_k||^2 of every iteration's projection residual, summed by
    the projection kernels (bulk-copy staged, per-thread, fused residual
    pass; packed and float masks), against the float64 oracle's value of the
    same residual map (pnp_sci_algo.py:640-645 for GAP, :808-809 for ADMM)
    on its own trajectory: the two trajectories differ by float32 rounding,
    so 1e-4 relative."""
    monkeypatch.setenv("SCI_FUSED_PROJ", "1" if fused else "0")
    H, W, B, iters = 64, 96, 8, 10
    orig, mask, meas = sci.datasets.video_config(H, W, B, noise_rel=0.01)
    msum = mask.sum(axis=2)
    msum[msum == 0] = 1
    op = sci.MaskOperator(mask)
    y = _dev.plane(meas)
    s = sci.Solver(op, kind, iters, 1.0, 0.1, 5, accelerate=acc, resid_norm=True,
                   use_bits=bits)
    s.run(y)
    rn = s.resid_norms()
    ref = []
    A = lambda v: port.A_(v, mask)       # noqa: E731
    At = lambda r: port.At_(r, mask)     # noqa: E731
    if kind == "gap":
        port.gap_denoise(meas, msum, A, At, _lambda=1, accelerate=acc, iter_max=iters,
                         tv_weight=0.1, tv_iter_max=5, x0=At(meas), show_iqa=False, resid=ref)
    else:
        port.admm_denoise(meas, msum, A, At, _lambda=1, gamma=0.01, iter_max=iters,
                          tv_weight=0.1, tv_iter_max=5, x0=At(meas), show_iqa=False,
                          resid=ref)
    assert len(ref) == iters
    np.testing.assert_allclose(rn, ref, rtol=1e-4)
    # without the option the solver records nothing and computes the same x
    plain = sci.Solver(op, kind, iters, 1.0, 0.1, 5, accelerate=acc, use_bits=bits)
    assert torch.equal(plain.run(y), s.x)
    with pytest.raises(ValueError):
        plain.resid_norms()


@pytest.mark.parametrize("shape,cpl", [((64, 96, 8), None), ((72, 1040, 24), None),
                                       ((40, 128, 12), "2"), ((33, 1032, 5), "4")])
@pytest.mark.parametrize("with_orig", [False, True])
def test_fused_admm_iteration(monkeypatch, shape, cpl, with_orig):
    """ADMM as residual pass + TV pass with the projection applied on load
    (the default with a packed mask) against the projection-kernel loop
    (SCI_ADMM_FUSED=0): the same iteration re-associated (the TV input
    formed as theta + lambda (r phi) instead of x - b), so equal to float32
    rounding -- 1e-5 relative L2 after 12 iterations with gammas and an
    annealed weight -- and the same per-iteration PSNR and residual norms to
    1e-4 relative."""
    if cpl is not None:
        monkeypatch.setenv("SCI_TV_CPL", cpl)
    orig, mask, meas = sci.datasets.video_config(*shape, noise_rel=0.01)
    op = sci.MaskOperator(mask)
    y = _dev.plane(meas)
    o = _dev.planar(orig) if with_orig else None
    iters = 12
    gam = np.linspace(0.01, 0.02, iters).astype(np.float32)
    w = np.array([0.2 * 0.25 ** (k / (iters - 1)) for k in range(iters)], np.float32)
    runs = []
    for fused in ("1", "0"):
        monkeypatch.setenv("SCI_ADMM_FUSED", fused)
        s = sci.Solver(op, "admm", iters, 1.0, w, 5, gammas=gam, resid_norm=True)
        x = s.run(y, orig=o).clone()
        runs.append((x, s.resid_norms(), s.psnr_all() if with_orig else None))
    (xa, ra, pa), (xb, rb, pb) = runs
    rel = float(torch.linalg.vector_norm(xa - xb) / torch.linalg.vector_norm(xb))
    assert rel < 1e-5, rel
    assert np.allclose(ra, rb, rtol=1e-4, atol=0)
    if with_orig:
        assert np.allclose(pa, pb, rtol=0, atol=1e-3)
