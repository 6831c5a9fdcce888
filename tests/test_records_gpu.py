"""Training-record extraction (nmg_extract_records) against the oracle's
restatement of generate_training_data (train.cu:14-67): seeded per-pixel
radiance records with delta vertices, throughputs below 1e-5, NaNs and zero
pdfs; a strided training-pixel grid; both input modes; the device count
feeding a training step; capacity overflow."""
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
        rec["thp"].append(thp)
        rec["L"].append(rng.lognormal(0, 1, (n, 3)).astype(np.float32))
        pos = rng.uniform(-2, 3, (n, 3)).astype(np.float32)
        pos[rng.random(n) < 0.01, 1] = np.nan
        rec["pos"].append(pos)
        dr = np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32)
        dr[rng.random(n) < 0.01, 0] = np.nan
        rec["dir"].append(dr)
        wp = rng.uniform(0.01, 2, n).astype(np.float32)
        wp[rng.random(n) < 0.02] = 0.0
        rec["wi_pdf"].append(wp)
        rec["bsdf_pdf"].append(rng.uniform(0.01, 2, n).astype(np.float32))
        rec["mis_weight"].append(rng.uniform(0, 1, n).astype(np.float32))
        rec["delta"].append((rng.random(n) < 0.1).astype(np.uint8))
        rec["bsdf_val"].append(rng.uniform(0, 1, (n, 3)).astype(np.float32))
        rec["wo"].append(np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32))
        rec["normal"].append(np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32))
        rec["roughness"].append(rng.uniform(0, 1, n).astype(np.float32))
    cur = rng.integers(0, depth + 1, n).astype(np.uint32)
    return rec, cur


def sort_rows(a):
    return a[np.lexsort(a.T[::-1])]


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
    got = sort_rows(np.concatenate([r.cpu().numpy()[:n], x.cpu().numpy()[:n]], 1).astype(np.float64))
    want = sort_rows(np.concatenate([r64, x64], 1))
    assert np.allclose(got, want, rtol=2e-6, atol=2e-6)
    # the count feeds a training step directly
    stats = f.train_step(x, r, count=cnt).cpu().numpy()
    assert np.all(np.isfinite(stats))
    # capacity below the record count: the count still reports every record, only `capacity` rows are written
    x2, r2, cnt2 = f.extract_records(dev, torch.from_numpy(cur.view(np.int32)).cuda(), OFFSET, STRIDE, TRAIN_RES, RES,
                                     capacity=100)
    assert int(cnt2.item()) == n and x2.shape[0] == 100
    f.check_errors()
    f.close()
