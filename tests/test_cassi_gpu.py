"""Spectral (CASSI) operators and GAP-TV on the GPU against the oracle.

The cube is 256 x 256 x 28 with smooth spectra, one Bernoulli(0.5)
aperture, a 2-pixel dispersion per band onto a 256 x 310 detector and 80
GAP-TV iterations (the spectral workload); the oracle is the reference's
own GAP loop (bit-exact numpy port) with the restated CASSI operators.
"""
import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev
from oracle import cassi as oc
from oracle import reference_port as port

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("H,W,L,step", [(8, 12, 3, 2), (37, 50, 28, 2), (64, 61, 9, 1),
                                        (20, 16, 5, 3)])
def test_cassi_operators(H, W, L, step):
    rng = np.random.default_rng(H + W + L)
    x = rng.random((H, W, L))
    phi = (rng.random((H, W)) < 0.5).astype(np.float64)
    phi[0, 0] = 0.37
    op = sci.CassiOperator(phi, L, step)
    y = op.forward(x)
    assert y.shape == (H, W + step * (L - 1))
    assert rel(y, oc.cassi_A(x, phi, step)) < 1e-6
    r = rng.standard_normal(y.shape)
    xt = op.adjoint(r)
    assert rel(xt, oc.cassi_At(r, phi, L, step)) < 1e-6
    lhs = float(np.sum(y.astype(np.float64) * r))
    rhs = float(np.sum(x * xt.astype(np.float64)))
    assert abs(lhs - rhs) <= 1e-5 * np.abs(y).sum() * np.abs(r).max()
    np.testing.assert_allclose(op.phisum.cpu().numpy(), oc.cassi_phisum(phi, L, step), rtol=1e-6)


def cassi_problem(iters_seed=0):
    cube = sci.datasets.spectral_cube(256, 256, 28, seed=iters_seed)
    phi = sci.datasets.bernoulli_mask(256, 256, 1, seed=1)[..., 0]
    y = oc.cassi_A(cube, phi, 2)
    return cube, phi, y


def test_cassi_gap_tv_matches_oracle():
    cube, phi, y = cassi_problem()
    L, iters = 28, 80
    ps = oc.cassi_phisum(phi, L, 2)
    A = lambda x: oc.cassi_A(x, phi, 2)  # noqa: E731
    At = lambda r: oc.cassi_At(r, phi, L, 2)  # noqa: E731
    ref, rpsnr, _, rall = port.gap_denoise(y, ps, A, At, _lambda=1, accelerate=True,
                                           iter_max=iters, tv_weight=0.05, tv_iter_max=5,
                                           X_orig=cube)
    Ag, Atg = sci.make_cassi_ops(phi, L, 2)
    x, psnr_, ssim_, pall = sci.gap_denoise(y, ps, Ag, Atg, _lambda=1, accelerate=True,
                                            iter_max=iters, tv_weight=0.05, tv_iter_max=5,
                                            X_orig=cube)
    r = rel(x, ref)
    print("CASSI 256x256x28, 80 it: rel L2 %.3e, PSNR %.3f vs %.3f" % (r, np.mean(psnr_),
                                                                       np.mean(rpsnr)))
    assert r < 1e-4
    assert np.max(np.abs(np.array(pall) - np.array(rall))) < 1e-2
    assert abs(np.mean(psnr_) - np.mean(rpsnr)) < 1e-2


def test_cassi_admm_plugin_path():
    """ADMM with the CASSI callables goes through the plug-in loop."""
    cube, phi, y = cassi_problem()
    cube, y = cube[:64, :64, :8], None
    phi = phi[:64, :64]
    L = 8
    y = oc.cassi_A(cube, phi, 2)
    ps = oc.cassi_phisum(phi, L, 2)
    A = lambda x: oc.cassi_A(x, phi, 2)  # noqa: E731
    At = lambda r: oc.cassi_At(r, phi, L, 2)  # noqa: E731
    ref = port.admm_denoise(y, ps, A, At, gamma=0.01, iter_max=10, tv_weight=0.05,
                            tv_iter_max=5)[0]
    Ag, Atg = sci.make_cassi_ops(phi, L, 2)
    x = sci.admm_denoise(y, ps, Ag, Atg, gamma=0.01, iter_max=10, tv_weight=0.05,
                         tv_iter_max=5)[0]
    assert rel(x, ref) < 1e-4


@pytest.mark.parametrize("accelerate", [True, False])
def test_cassi_row_projection_and_graph_are_bitwise_equal(monkeypatch, accelerate):
    """The row-fused projection (residual row in shared memory; 512 or 1024
    threads per row) against the detector-grid +
    cube-grid kernel pair, and the captured graph (first run and replay)
    against direct launches: identical solves."""
    cube, phi, y = cassi_problem()
    op = sci.CassiOperator(phi, 28, 2)
    yd = torch.from_numpy(y).float().to(op.dev)
    out = []
    for rows, graph in (("1", True), ("1", False), ("1024", False), ("0", False), ("0", True)):
        if rows == "1024":
            monkeypatch.setenv("SCI_CASSI_ROWT", rows)
            rows = "1"
        monkeypatch.setenv("SCI_CASSI_ROWS", rows)
        s = sci.CassiSolver(op, 12, 1.0, 0.05, 5, accelerate=accelerate, use_graph=graph)
        out.append(s.run(yd).clone())
        if graph:
            out.append(s.run(yd).clone())  # replay of the cached graph
    for o in out[1:]:
        assert torch.equal(o, out[0])
