"""Training-record extraction (nmg_extract_records) against the reference's
own generate_training_data (train.cu:14-67) and the oracle's FP32
restatement of it: seeded per-pixel radiance records with delta vertices,
throughputs below and exactly at 1e-5, NaN positions / directions / outgoing
directions / pdfs / MIS weights / radiance, NaN and Inf BSDF values, zero
pdfs; a strided training-pixel grid; both input modes; the device count
feeding a training step; capacity overflow.

Tolerances: the kept-record set, the GuidedOutput rows (NaN radiance
included) and the normalised positions bit for bit; the inputs computed
through sin/cos/exp (device functions against the host libm the reference
was run with) within 2 ulp of 1.0, their scale."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES = (61, 37)
OFFSET, STRIDE = (1, 2), (3, 2)
TRAIN_RES = (21, 19)  # the last row/column of the grid falls outside the image


def make_records(rng, depth=8):
    n = RES[0] * RES[1]
    rec = {k: [] for k in ("L", "thp", "pos", "dir", "wi_pdf", "bsdf_pdf", "mis_weight", "delta", "bsdf_val", "wo",
                           "normal", "roughness")}
    for _ in range(depth):
        thp = rng.uniform(0, 1, (n, 3)).astype(np.float32)
        thp[rng.random((n, 3)) < 0.05] = 5e-6
        thp[rng.random((n, 3)) < 0.03] = np.float32(1e-5)
        rec["thp"].append(thp)
        L = rng.lognormal(0, 1, (n, 3)).astype(np.float32)
        L[rng.random(n) < 0.01, 2] = np.nan
        rec["L"].append(L)
        pos = rng.uniform(-2, 3, (n, 3)).astype(np.float32)
        pos[rng.random(n) < 0.01, 1] = np.nan
        rec["pos"].append(pos)
        dr = np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32)
        dr[rng.random(n) < 0.01, 0] = np.nan
        rec["dir"].append(dr)
        wp = rng.uniform(0.01, 2, n).astype(np.float32)
        wp[rng.random(n) < 0.02] = 0.0
        wp[rng.random(n) < 0.01] = np.nan
        rec["wi_pdf"].append(wp)
        rec["bsdf_pdf"].append(rng.uniform(0.01, 2, n).astype(np.float32))
        mw = rng.uniform(0, 1, n).astype(np.float32)
        mw[rng.random(n) < 0.01] = np.nan
        rec["mis_weight"].append(mw)
        rec["delta"].append((rng.random(n) < 0.1).astype(np.uint8))
        bv = rng.uniform(0, 1, (n, 3)).astype(np.float32)
        bv[rng.random(n) < 0.02, 0] = np.nan  # kept: only the stored radiance becomes NaN
        bv[rng.random(n) < 0.02, 1] = np.inf
        rec["bsdf_val"].append(bv)
        wo = np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32)
        wo[rng.random(n) < 0.02, 0] = np.nan  # dropped: NaN warped outgoing direction
        rec["wo"].append(wo)
        rec["normal"].append(np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32))
        rec["roughness"].append(rng.uniform(0, 1, n).astype(np.float32))
    cur = rng.integers(0, depth + 1, n).astype(np.uint32)
    return rec, cur


def by_position(x, r):
    """Rows in the order of their normalised positions (exact and distinct): the device appends in no
    fixed order."""
    o = np.lexsort(x[:, 2::-1].T)
    return x[o], r[o]


def assert_records_equal(x, r, x_want, r_want):
    x, r = by_position(x, r)
    x_want, r_want = by_position(x_want, r_want)
    assert np.array_equal(r, r_want, equal_nan=True)
    assert np.array_equal(x[:, :3], x_want[:, :3])
    assert np.abs(x[:, 3:] - x_want[:, 3:]).max() <= 2 * np.spacing(np.float32(1))


@pytest.mark.parametrize("preset", [0, 1], ids=["reference-inputs", "sh-normal-inputs"])
def test_extract_records_vs_oracle(nmg, oracle, preset):
    import torch
    rng = np.random.default_rng(40 + preset)
    rec, cur = make_records(rng)
    aabb = [-2, -2, -2, 3, 3, 3]
    f = nmg.GuidingField(nmg.config(preset, aabb=aabb), max_batch=1 << 14)
    dev = [{k: torch.from_numpy(np.ascontiguousarray(v[d])).cuda() for k, v in rec.items()} for d in range(8)]
    x, r, cnt = f.extract_records(dev, torch.from_numpy(cur.view(np.int32)).cuda(), OFFSET, STRIDE, TRAIN_RES, RES,
                                  capacity=1 << 14)
    n = int(cnt.item())
    x64, r64 = oracle.extract_records(rec, cur, OFFSET, STRIDE, TRAIN_RES, RES, aabb, input_mode=f.cfg.input_mode,
                                      selection=bool(f.cfg.selection))
    assert n == len(x64) and n > 1000
    assert np.isnan(r64[:, 2:5]).any() and np.isinf(r64[:, 2:5]).any()
    assert_records_equal(x.cpu().numpy()[:n], r.cpu().numpy()[:n], x64, r64)
    # the count feeds a training step directly (the records the reference keeps with a NaN or Inf
    # radiance give a non-finite loss term there too; the step's gradient drops them as the
    # reference's NaN/Inf gradient check does)
    stats = f.train_step(x, r, count=cnt).cpu().numpy()
    assert stats.shape == (2,)
    # capacity below the record count: the count still reports every record, only `capacity` rows are written
    x2, r2, cnt2 = f.extract_records(dev, torch.from_numpy(cur.view(np.int32)).cuda(), OFFSET, STRIDE, TRAIN_RES, RES,
                                     capacity=100)
    assert int(cnt2.item()) == n and x2.shape[0] == 100
    f.check_errors()
    f.close()


def test_extract_records_vs_reference_kernel(nmg):
    """The reference's own generate_training_data, run on the same inputs (tests/golden/train_cu_golden.npz,
    written by tests/golden/make_golden.py), against nmg_extract_records."""
    import torch
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "train_cu_golden.npz")))
    keys = ("L", "thp", "pos", "dir", "wi_pdf", "bsdf_pdf", "mis_weight", "delta", "bsdf_val", "wo", "normal",
            "roughness")
    depth = g["rec_L"].shape[0]
    f = nmg.GuidingField(nmg.config(nmg.PRESET_REFERENCE, aabb=[float(v) for v in g["aabb"]]), max_batch=4096)
    dev = [{k: torch.from_numpy(np.ascontiguousarray(g["rec_" + k][d])).cuda() for k in keys} for d in range(depth)]
    cur = torch.from_numpy(g["cur_depth"].view(np.int32)).cuda()
    x, r, cnt = f.extract_records(dev, cur, tuple(g["offset"]), tuple(g["stride"]), tuple(g["train_res"]),
                                  tuple(g["res"]), capacity=4096)
    n = int(cnt.item())
    assert n == len(g["rec_x"])
    assert_records_equal(x.cpu().numpy()[:n], r.cpu().numpy()[:n], g["rec_x"], g["rec_out"])
    f.check_errors()
    f.close()
