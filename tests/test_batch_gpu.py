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
    """The per-phase launches' bulk-copy staged batch projection against
    their per-thread shared-memory kernel: identical results after 6
    iterations."""
    shapes = [(64, 64, 8, 0.5), (40, 48, 4, 0.7), (33, 200, 32, 0.45), (96, 256, 12, 0.6),
              (300, 260, 24, 0.5)]
    data = make_items(shapes, seed=5)
    monkeypatch.setenv("SCI_BATCH_QUEUE", "0")
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


def _batch_runs(data, monkeypatch, configs, iters=7, accelerate=True):
    """Solves the batch once per (env, iters_per_launch, cpl) configuration."""
    out = []
    for env, ipl, cpl in configs:
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        bs = sci.BatchSolver([d[2] for d in data], [d[1] for d in data], iters=iters,
                             tv_weight=0.1, accelerate=accelerate, autotune=False)
        bs.iters_per_launch = ipl
        for i in range(len(bs.xs)):
            # cpl "mix": 2 and 4 columns per lane on alternate items, so that
            # warps of one block run both widths
            bs.items[i].cpl = (2 if i % 2 else 4) if cpl == "mix" else cpl
        out.append([x.clone() for x in bs.run()])
        for k in env:
            monkeypatch.delenv(k)
    return out


@pytest.mark.parametrize("accelerate", [True, False])
def test_batch_work_queue_equals_per_phase_launches(monkeypatch, accelerate):
    """The persistent work-queue launches (any number of iterations per
    launch, either TV column width) against one launch per phase: the same
    per-pixel arithmetic, bit-identical items."""
    shapes = [(64, 64, 8, 0.5), (40, 48, 4, 0.7), (33, 200, 32, 0.45), (96, 256, 12, 0.6),
              (300, 260, 24, 0.5), (128, 1024, 16, 0.5)]
    data = make_items(shapes, seed=11)
    runs = _batch_runs(data, monkeypatch,
                       [({"SCI_BATCH_QUEUE": "0"}, 0, 0), ({}, 0, 0), ({}, 1, 0), ({}, 3, 0),
                        ({}, 0, 2), ({}, 2, 2), ({}, 0, "mix"), ({}, 1, "mix")],
                       accelerate=accelerate)
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert torch.equal(a, b)


def test_batch_work_queue_wait_gives_up_and_context_stays_usable():
    """The bounded wait of the work queue gives up on a count that nothing
    raises, sets status bit 1, and the next batch solve is valid."""
    from sci_algorithms_gb300._lib import call
    import ctypes
    ws = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    st = ctypes.c_uint(0)
    call("sci_device_status", ctypes.byref(st), 1)
    call("sci_batch_selftest_queue_wait", 2000, ws.data_ptr(), ws.numel(),
         _dev.stream_handle())
    torch.cuda.synchronize()
    call("sci_device_status", ctypes.byref(st), 1)
    assert st.value & 2
    call("sci_device_status", ctypes.byref(st), 0)
    assert st.value == 0
    data = make_items([(64, 64, 8, 0.5), (40, 48, 4, 0.7)], seed=3)
    bs = sci.BatchSolver([d[2] for d in data], [d[1] for d in data], iters=5, autotune=False)
    res = [x.clone() for x in bs.run()]
    for i, (orig, mask, meas) in enumerate(data):
        s = sci.Solver(bs.ops[i], "gap", 5, 1.0, 0.1, 5, use_graph=False)
        bs0 = sci.BatchSolver([meas], [mask], iters=0, autotune=False)
        assert torch.equal(res[i], s.run(bs.ys[i], x0=bs0.run()[0].clone()))
    call("sci_device_status", ctypes.byref(st), 0)
    assert st.value == 0


def test_batch_config4_every_item_matches_single_solver():
    """The 64-item uneven batch (H = W in 128..1024, B in 8..32, 50
    iterations, autotuned), every item against the single-measurement solver
    from the same start point, and one 1024 x 1024 x 32 item against the
    float64 C oracle."""
    meas, masks = [], []
    for orig, mask, y in sci.datasets.batch_config(64, seed=0):
        meas.append(y)
        masks.append(mask)
        del orig
    bs = sci.BatchSolver(meas, masks, iters=50, tv_weight=0.1, autotune=True)
    assert set(bs.columns_per_lane()) <= {2, 4}
    res = [x.clone() for x in bs.run()]
    x0s = [x.clone() for x in sci.BatchSolver(meas, masks, iters=0, autotune=False).run()]
    big = None
    for i in range(len(meas)):
        s = sci.Solver(bs.ops[i], "gap", 50, 1.0, 0.1, 5)
        ref = s.run(bs.ys[i], x0=x0s[i])
        assert torch.equal(res[i], ref), i
        del s
        if masks[i].shape == (1024, 1024, 32) and big is None:
            big = i
    if big is not None:
        mask, y = masks[big], meas[big]
        msum = mask.sum(axis=2)
        msum[msum == 0] = 1
        x0 = c_oracle.planar(mask * (y / msum)[..., None])
        ref, _ = c_oracle.gap_tv(y, c_oracle.planar(mask), msum, x0, 50, 1.0, 0.1)
        r = np.linalg.norm(res[big].cpu().numpy() - ref) / np.linalg.norm(ref)
        assert r < 1e-4, r
