"""Batched uneven GAP-TV: every item equals the single-measurement solver,
and small items match the float64 oracle."""
import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev
from oracle import c_oracle

pytestmark = pytest.mark.gpu


def make_items(shapes, seed=0):
    out = []
    for i, (H, W, B, p) in enumerate(shapes):
        out.append(sci.datasets.video_config(H, W, B, p=p, seeds=(seed + 3 * i, seed + 3 * i + 1,
                                                                   seed + 3 * i + 2)))
    return out


@pytest.mark.parametrize("autotune", [False, True])
def test_batch_matches_single_solver(autotune):
    shapes = [(64, 64, 8, 0.5), (128, 96, 16, 0.3), (40, 48, 4, 0.7), (256, 128, 24, 0.5),
              (33, 200, 32, 0.45), (96, 256, 12, 0.6)]
    data = make_items(shapes)
    iters = 9
    bs = sci.BatchSolver([d[2] for d in data], [d[1] for d in data], iters=iters, tv_weight=0.1,
                         autotune=autotune)
    bs0 = sci.BatchSolver([d[2] for d in data], [d[1] for d in data], iters=0, autotune=False)
    x0 = [x.clone() for x in bs0.run()]  # At(y / Phi_sum) as the batch forms it
    res = [x.clone() for x in bs.run()]
    for i, (orig, mask, meas) in enumerate(data):
        op = bs.ops[i]
        s = sci.Solver(op, "gap", iters, 1.0, 0.1, 5, use_graph=False)
        ref = s.run(bs.ys[i], x0=x0[i])
        assert float((res[i] - ref).abs().max()) < 1e-6, i
    # replaying the captured graph gives the same result
    again = bs.run()
    for a, b in zip(res, again):
        assert torch.equal(a, b)


@pytest.mark.parametrize("accelerate", [True, False])
def test_batch_bulk_copy_projection_is_bitwise_equal(monkeypatch, accelerate):
    """The bulk-copy staged batch projection (the default) against the
    per-thread shared-memory kernel: identical results after 6 iterations."""
    shapes = [(64, 64, 8, 0.5), (40, 48, 4, 0.7), (33, 200, 32, 0.45), (96, 256, 12, 0.6),
              (300, 260, 24, 0.5)]
    data = make_items(shapes, seed=5)
    runs = []
    for tma in ("1", "0"):
        monkeypatch.setenv("SCI_PROJ_TMA", tma)
        bs = sci.BatchSolver([d[2] for d in data], [d[1] for d in data], iters=6, tv_weight=0.1,
                             accelerate=accelerate, autotune=False)
        runs.append([x.clone() for x in bs.run()])
    for a, b in zip(*runs):
        assert torch.equal(a, b)


def test_batch_against_oracle():
    shapes = [(48, 64, 8, 0.5), (64, 40, 6, 0.4)]
    data = make_items(shapes, seed=7)
    iters = 12
    bs = sci.BatchSolver([d[2] for d in data], [d[1] for d in data], iters=iters, tv_weight=0.15)
    res = bs.run()
    for i, (orig, mask, meas) in enumerate(data):
        msum = mask.sum(axis=2)
        msum[msum == 0] = 1
        x0 = c_oracle.planar(mask * (meas / msum)[..., None])
        ref, _ = c_oracle.gap_tv(meas, c_oracle.planar(mask), msum, x0, iters, 1.0, 0.15)
        r = np.linalg.norm(res[i].cpu().numpy() - ref) / np.linalg.norm(ref)
        assert r < 1e-4, (i, r)


def test_batch_rejects_bad_items():
    data = make_items([(16, 18, 4, 0.5)])
    with pytest.raises(Exception, match="W % 4"):
        sci.BatchSolver([data[0][2]], [data[0][1]], iters=2)
