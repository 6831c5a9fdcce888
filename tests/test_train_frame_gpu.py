"""One frame's training on its radiance records (nmg_train_frame), the
reference's trainStep (integrator.cpp:650-701): record compaction into vertex
ids, then batches sized on the device, the fused training kernel computing
each record's network input and GuidedOutput in its load stage.

Checked against the unfused route on the same batch -- the records
nmg_extract_records writes, put in the order of train_frame's vertex ids,
trained by nmg_train_step -- on the plain FP32 and the fused BF16 path: the
same gradient up to the order of the floating-point atomics (1e-5 of the
largest component for FP32, 1e-3 for BF16, whose grid gradient is summed by
float atomics in a different order), the same mean loss (1e-6 relative).
Also the batch plan: batch i holds min(N - i B, B) records rounded down to a
multiple of 128, batches below min_batch take no optimiser step, and a
capacity below N caps the records trained."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES = (97, 53)
DEPTH = 6
AABB = [-2, -2, -2, 3, 3, 3]


def make_records(rng):
    n = RES[0] * RES[1]
    rec = {k: [] for k in ("L", "thp", "pos", "dir", "wi_pdf", "bsdf_pdf", "mis_weight", "delta", "bsdf_val", "wo",
                           "normal", "roughness")}

    def ang():
        return np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)], 1).astype(np.float32)

    for _ in range(DEPTH):
        rec["thp"].append(rng.uniform(0.05, 1, (n, 3)).astype(np.float32))
        rec["L"].append(rng.lognormal(0, 1, (n, 3)).astype(np.float32))
        rec["pos"].append(rng.uniform(-2, 3, (n, 3)).astype(np.float32))
        rec["dir"].append(ang())
        wp = rng.uniform(0.01, 2, n).astype(np.float32)
        wp[rng.random(n) < 0.02] = 0.0
        rec["wi_pdf"].append(wp)
        rec["bsdf_pdf"].append(rng.uniform(0.01, 2, n).astype(np.float32))
        rec["mis_weight"].append(rng.uniform(0, 1, n).astype(np.float32))
        rec["delta"].append((rng.random(n) < 0.1).astype(np.uint8))
        rec["bsdf_val"].append(rng.uniform(0, 1, (n, 3)).astype(np.float32))
        wo = ang()
        wo[rng.random(n) < 0.01, 0] = np.nan
        rec["wo"].append(wo)
        rec["normal"].append(ang())
        rec["roughness"].append(rng.uniform(0, 1, n).astype(np.float32))
    cur = rng.integers(0, DEPTH + 1, n).astype(np.uint32)
    return rec, cur


def to_device(rec, cur):
    import torch
    dev = [{k: torch.from_numpy(np.ascontiguousarray(v[d])).cuda() for k, v in rec.items()} for d in range(DEPTH)]
    return dev, torch.from_numpy(cur.view(np.int32)).cuda()


def full_grid():
    return (0, 0), (1, 1), RES, RES


@pytest.mark.parametrize("path", [0, 1], ids=["fp32", "bf16"])
def test_single_batch_equals_extract_then_train(nmg, oracle, path):
    import torch
    rng = np.random.default_rng(71)
    rec, cur = make_records(rng)
    dev, dcur = to_device(rec, cur)
    cfg = nmg.config(nmg.PRESET_HASHGRID, path=path, aabb=AABB)
    B = 1 << 15
    f1 = nmg.GuidingField(cfg, max_batch=B)
    f2 = nmg.GuidingField(cfg, max_batch=B)
    cap = RES[0] * RES[1] * DEPTH
    ids, cnt, stats = f1.train_frame(dev, dcur, *full_grid(), capacity=cap, batch_size=B, max_batches=1,
                                     min_batch=0)
    n = int(cnt.item())
    nb = n - n % 128
    assert 10000 < n < B and f1.step == 1
    # the same records through nmg_extract_records, reordered to train_frame's vertex ids
    x, r, cnt2 = f2.extract_records(dev, dcur, *full_grid(), capacity=cap)
    assert int(cnt2.item()) == n
    xh = x.cpu().numpy()[:n]
    _, _, verts = oracle.extract_records(rec, cur, *full_grid(), AABB, input_mode=cfg.input_mode,
                                         selection=bool(cfg.selection), return_vertex=True)
    xo, _ = oracle.extract_records(rec, cur, *full_grid(), AABB, input_mode=cfg.input_mode,
                                   selection=bool(cfg.selection))
    pixels = RES[0] * RES[1]
    # the normalised position is bit-exact on the device and in the oracle: it identifies the record
    vid_of_pos = {xo[i, :3].tobytes(): int(verts[i, 1]) * pixels + int(verts[i, 0]) for i in range(len(xo))}
    row_of_vid = {vid_of_pos[xh[i, :3].tobytes()]: i for i in range(n)}
    order = [row_of_vid[int(v)] for v in ids.cpu().numpy().view(np.uint32)[:nb]]
    idx = torch.tensor(order, device="cuda")
    st2 = f2.train_step(x[:n][idx].contiguous(), r[:n][idx].contiguous())
    g1, g2 = f1.get_gradients().cpu().numpy(), f2.get_gradients().cpu().numpy()
    tol = (1e-5 if path == 0 else 1e-3) * np.abs(g2).max()
    assert np.abs(g1 - g2).max() <= tol
    s1, s2 = stats.cpu().numpy()[0], st2.cpu().numpy()
    assert abs(s1[0] - s2[0]) <= 1e-6 * abs(s2[0])
    f1.check_errors()
    f1.close()
    f2.close()


@pytest.mark.parametrize("path", [0, 1], ids=["fp32", "bf16"])
def test_batch_plan_and_empty_batches(nmg, path):
    import torch
    rng = np.random.default_rng(72)
    rec, cur = make_records(rng)
    dev, dcur = to_device(rec, cur)
    cfg = nmg.config(nmg.PRESET_HASHGRID, path=path, aabb=AABB)
    B = 2048
    f = nmg.GuidingField(cfg, max_batch=B)
    cap = RES[0] * RES[1] * DEPTH
    ids, cnt, stats = f.train_frame(dev, dcur, *full_grid(), capacity=cap, batch_size=B, max_batches=12,
                                    min_batch=1000)
    n = int(cnt.item())
    want = []
    for i in range(12):
        c = min(max(n - i * B, 0), B)
        c -= c % 128
        want.append(c if c >= 1000 else 0)
    active = sum(1 for c in want if c > 0)
    assert 0 < active < 12 and f.step == active
    st = stats.cpu().numpy()
    assert np.all(st[:active, 1] > 0) and np.all(st[active:] == 0)
    # no batch reaches min_batch: no optimiser step, parameters unchanged
    p0 = f.get_params(0).clone()
    f.train_frame(dev, dcur, *full_grid(), capacity=cap, batch_size=B, max_batches=2, min_batch=B + 128)
    assert f.step == active and torch.equal(f.get_params(0), p0)
    # a capacity below the record count caps the records trained: one full batch of the first B ids
    _, cnt3, st3 = f.train_frame(dev, dcur, *full_grid(), capacity=B + 100, batch_size=B, max_batches=4,
                                 min_batch=0)
    assert int(cnt3.item()) == n and f.step == active + 1
    assert np.all(st3.cpu().numpy()[1:] == 0)
    f.check_errors()
    f.close()
