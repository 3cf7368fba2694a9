"""GPU Chambolle TV against the oracle restatement (scikit-image 0.16 rule).

Covers the single-pass pipeline (n_iter_max <= 5), multi-pass runs that
carry the dual field through the workspace, the speculative stop test and
its re-run, odd widths (scalar path), frames smaller than one band, and
2048-wide frames with many bands and row chunks.
"""
import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev
from oracle.tv_chambolle import tv_chambolle_frames, denoise_tv_chambolle as tv_ref
from oracle import c_oracle

pytestmark = pytest.mark.gpu

# float32 pipeline (approximate sqrt / reciprocal) vs float64 oracle, on
# images with values in [0, 1]: absolute error per pixel
ATOL = 2e-5


def smooth_frames(H, W, F, seed):
    rng = np.random.default_rng(seed)
    base = sci.datasets.video_scene(H, W, F, seed=seed)
    return np.clip(base + 0.05 * rng.standard_normal((H, W, F)), 0, 1)


def run_gpu(f_hwb, weight, K, eps=2e-4, resid=False):
    fp = _dev.planar(f_hwb)
    steps = torch.zeros(fp.shape[0], dtype=torch.int32, device=fp.device)
    energy = torch.zeros((fp.shape[0], K, 2), dtype=torch.float64, device=fp.device)
    r = torch.empty_like(fp) if resid else None
    u = sci.tv_frames(fp, weight, K, eps, resid=r, steps=steps, energy=energy)
    torch.cuda.synchronize()
    return (_dev.unplanar(u, f_hwb), steps.cpu().numpy(), energy.cpu().numpy(),
            None if r is None else _dev.unplanar(r, f_hwb))


@pytest.mark.parametrize("H,W,F", [(16, 16, 1), (37, 61, 3), (64, 128, 4), (130, 260, 2),
                                   (300, 500, 2), (256, 256, 8), (1, 8, 2), (5, 3, 2),
                                   (2, 129, 1), (200, 124, 3)])
@pytest.mark.parametrize("K", [1, 2, 3, 5])
def test_tv_single_pass_matches_oracle(H, W, F, K):
    f = smooth_frames(H, W, F, seed=H * 1000 + W + K)
    ref, steps_ref, _ = tv_chambolle_frames(f, 0.1, n_iter_max=K)
    u, steps, _, _ = run_gpu(f, 0.1, K)
    assert np.max(np.abs(u - ref)) < ATOL
    assert list(steps) == steps_ref


@pytest.mark.parametrize("K", [6, 9, 10, 13, 30])
def test_tv_multi_pass_and_early_stop(K):
    f = smooth_frames(96, 136, 6, seed=K)
    ref, steps_ref, _ = tv_chambolle_frames(f, 0.15, n_iter_max=K)
    u, steps, _, _ = run_gpu(f, 0.15, K)
    assert list(steps) == steps_ref
    assert np.max(np.abs(u - ref)) < ATOL * 2


def test_tv_early_stop_inside_single_pass():
    # a large eps makes the stop rule fire at k = 1..3 inside the 5-step pass
    f = smooth_frames(72, 80, 8, seed=5)
    for eps in (0.5, 0.2, 0.05, 0.02):
        ref, steps_ref, _ = tv_chambolle_frames(f, 0.2, eps=eps, n_iter_max=5)
        u, steps, _, _ = run_gpu(f, 0.2, 5, eps=eps)
        assert list(steps) == steps_ref, eps
        assert np.max(np.abs(u - ref)) < ATOL


def test_tv_energies_match_oracle():
    f = smooth_frames(64, 96, 3, seed=9)
    w, K = 0.1, 5
    _, steps_ref, e_ref = tv_chambolle_frames(f, w, n_iter_max=K)
    _, steps, en, _ = run_gpu(f, w, K)
    for b in range(3):
        for j in range(K - 1):  # E_{K-1} does not affect the result and is not formed
            e = (en[b, j, 0] + w * en[b, j, 1]) / (64 * 96)
            assert abs(e - e_ref[b][j]) <= 1e-5 * abs(e_ref[b][j])


def test_tv_constant_frames_unchanged_and_resid():
    f = np.full((50, 70, 3), 0.25)
    f[..., 1] = 0.0
    u, steps, _, r = run_gpu(f, 0.3, 5, resid=True)
    assert np.array_equal(u, f.astype(np.float32))
    assert np.all(r == 0)
    g = smooth_frames(50, 70, 3, seed=1)
    u, _, _, r = run_gpu(g, 0.3, 5, resid=True)
    assert np.max(np.abs(r - (u - g.astype(np.float32)))) < 1e-6


def test_tv_wide_frames_against_c_oracle():
    f = smooth_frames(2048, 2048, 2, seed=3)
    u, steps, _, _ = run_gpu(f, 0.1, 5)
    ref, csteps, _ = c_oracle.tv_chambolle(c_oracle.planar(f), 0.1, 5)
    assert list(steps) == list(csteps)
    assert np.max(np.abs(u - c_oracle.unplanar(ref))) < ATOL


def test_denoise_tv_chambolle_api():
    f = smooth_frames(40, 48, 4, seed=2)
    out = sci.denoise_tv_chambolle(f, 0.1, n_iter_max=5, multichannel=True)
    assert out.dtype == f.dtype and out.shape == f.shape
    assert np.max(np.abs(out - tv_ref(f, 0.1, n_iter_max=5, multichannel=True))) < ATOL
    g = f[..., 0].astype(np.float32)
    out2 = sci.denoise_tv_chambolle(g, 0.2, n_iter_max=4)
    assert out2.dtype == np.float32
    assert np.max(np.abs(out2 - tv_ref(g.astype(np.float64), 0.2, n_iter_max=4))) < ATOL
    t = torch.from_numpy(f).cuda()
    out3 = sci.denoise_tv_chambolle(t, 0.1, n_iter_max=5, multichannel=True)
    assert out3.is_cuda and torch.allclose(out3.double().cpu(), torch.from_numpy(out), atol=1e-6)
    with pytest.raises(NotImplementedError):
        sci.denoise_tv_chambolle(f, 0.1, multichannel=False)


# Frames wider than 512 columns run the register-lean single-pass kernel
# (sci_tv_slim.cuh); SCI_TV_SLIM=0 selects the generic pipeline.  The two
# perform the same float32 operations in the same order, so their frames are
# bit-identical and their stop steps equal.
SLIM_SHAPES = [(64, 1024, 3), (257, 516, 2), (130, 2048, 2), (33, 640, 5), (40, 520, 2),
               (200, 1028, 3), (7, 1536, 2)]


def _tv_env(monkeypatch, fp, weight, K, eps, slim, R=None):
    monkeypatch.setenv("SCI_TV_SLIM", slim)
    if R is None:
        monkeypatch.delenv("SCI_TV_R", raising=False)
    else:
        monkeypatch.setenv("SCI_TV_R", str(R))
    nf = fp.shape[0]
    steps = torch.zeros(nf, dtype=torch.int32, device=fp.device)
    energy = torch.zeros((nf, K, 2), dtype=torch.float64, device=fp.device)
    u = sci.tv_frames(fp, weight, K, eps, steps=steps, energy=energy)
    torch.cuda.synchronize()
    return u, steps.cpu().numpy(), energy.cpu().numpy()


@pytest.mark.parametrize("H,W,F", SLIM_SHAPES + [(64, 256, 3), (37, 62, 2), (300, 500, 2)])
@pytest.mark.parametrize("K", [2, 3, 4, 5])
@pytest.mark.parametrize("cpl", ["2", "4"])
def test_tv_slim_bitwise_equals_generic(H, W, F, K, cpl, monkeypatch):
    monkeypatch.setenv("SCI_TV_CPL", cpl)
    f = smooth_frames(H, W, F, seed=7 * H + W + K)
    fp = _dev.planar(f)
    u0, s0, e0 = _tv_env(monkeypatch, fp, 0.1, K, 2e-4, "0")
    u1, s1, e1 = _tv_env(monkeypatch, fp, 0.1, K, 2e-4, "1")
    assert torch.equal(u0, u1)
    assert list(s0) == list(s1)
    # the energy sums are float32 per lane and chunk (the two kernels may
    # chunk the rows differently), then float64
    np.testing.assert_allclose(e1, e0, rtol=1e-6, atol=0)


@pytest.mark.parametrize("H,W,F", [(64, 1024, 3), (257, 516, 2), (33, 640, 5)])
def test_tv_slim_matches_oracle(H, W, F, monkeypatch):
    f = smooth_frames(H, W, F, seed=H + W)
    ref, steps_ref, _ = tv_chambolle_frames(f, 0.1, n_iter_max=5)
    u, steps, _ = _tv_env(monkeypatch, _dev.planar(f), 0.1, 5, 2e-4, "1")
    assert np.max(np.abs(_dev.unplanar(u, f) - ref)) < ATOL
    assert list(steps) == steps_ref


@pytest.mark.parametrize("R", [8, 16, 29, 64])
def test_tv_slim_row_chunks_and_early_stop(R, monkeypatch):
    # forced chunk heights and stop rules that fire at steps 1..3 (the
    # re-run launch of the lean kernel)
    f = smooth_frames(150, 1032, 4, seed=R)
    fp = _dev.planar(f)
    for eps in (0.5, 0.2, 0.05, 0.02, 2e-4):
        ref, steps_ref, _ = tv_chambolle_frames(f, 0.2, eps=eps, n_iter_max=5)
        u1, s1, _ = _tv_env(monkeypatch, fp, 0.2, 5, eps, "1", R=R)
        u0, s0, _ = _tv_env(monkeypatch, fp, 0.2, 5, eps, "0", R=R)
        assert list(s1) == steps_ref, eps
        assert list(s0) == list(s1), eps
        assert torch.equal(u0, u1), eps
        assert np.max(np.abs(_dev.unplanar(u1, f) - ref)) < ATOL


@pytest.mark.parametrize("cpl,minbs", [("4", ("3", "4")), ("2", ("5", "6", "7"))])
def test_tv_slim_occupancy_variants(cpl, minbs, monkeypatch):
    # the register budgets of the lean kernel agree bit for bit
    monkeypatch.setenv("SCI_TV_CPL", cpl)
    f = smooth_frames(96, 2048, 3, seed=3)
    fp = _dev.planar(f)
    outs = []
    for mb in minbs:
        monkeypatch.setenv("SCI_SLIM_MINB", mb)
        for form in ("0", "1"):  # the dual field as p or as 4 p
            monkeypatch.setenv("SCI_TV_FORM", form)
            outs.append(_tv_env(monkeypatch, fp, 0.1, 5, 2e-4, "1"))
    for u, s, _ in outs[1:]:
        assert torch.equal(outs[0][0], u)
        assert list(outs[0][1]) == list(s)
