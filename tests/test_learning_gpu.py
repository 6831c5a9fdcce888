"""What the learned guide buys, and whether the fused BF16/FP16 paths learn as
well as the FP32 path.

Ground truth: the seeded 16^3-cell radiance field (each cell a 4-lobe vMF
mixture, kappa log-uniform on [1, 200]). Every training step draws a fresh
batch of 2^18 records from it on the GPU, as a renderer records new paths
each frame (50% of directions from the field, 50% uniform; radiance =
density x lognormal(0, 0.5)), on the same 64 planes as the evaluation
queries. Network: the hash-grid preset with 8 lobes, no learned selection,
Adam at learning rate 1e-3 for 3,000 steps.

At the reference's 1e-2 (common/configs/nn/base.json) the bias-free MLP can
drive every kappa logit far below the exp clamp within a few dozen steps,
after which the guide stays at the uniform density: with the same data this
happens or not depending on the seed, in every path (FP32, BF16, FP16) and
in an FP64 autograd model of the same network alike. At 1e-2 a precision
comparison therefore measures the chance of that collapse. At 3e-3 the
float-atomic order alone moves the KL after 1,000-3,000 steps by 1-4%
between two runs of the same path; at 1e-3 two runs agree within 0.3%
(measured KL after 3,000 steps: FP32 0.684 / 0.683, BF16 0.660 / 0.659,
FP16 0.673).

The quality measure is KL(g || q) = E_{w~g}[log g(w) - log q(w)] per query,
estimated on held-out queries by sampling w from the ground truth g, with q
the guide's pdf (nmg_pdf, inference/EMA weights, cosine product off because
the ground truth carries no cosine factor). Reference points without a
network: the uniform sphere and the cosine lobe around the normal.

(Training on a small fixed pool of batches instead lets the 12.6 M-parameter
hash grid memorise individual records: the training loss keeps falling while
the KL on new directions rises. Fresh records avoid that, as in rendering.)
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 3000
BATCH = 1 << 18
LR = 1e-3
N_EVAL = 1 << 16
EVAL_SEED = 99


def _train(nmg, synth, path, steps=STEPS, seed=7272):
    import torch
    cfg = nmg.config(1, path=path, selection=0, cosine_aware=0, learning_rate=LR)
    f = nmg.GuidingField(cfg, max_queries=N_EVAL, max_batch=BATCH)
    gt = synth.TrainField(seed=seed)
    src = synth.TorchTrainSource(gt, seed=seed + 1, plane_seed=EVAL_SEED + 1)
    stats = torch.zeros(2, device="cuda", dtype=torch.float64)
    for _ in range(steps):
        x, rec = src(BATCH)
        f.train_step(x, rec, stats=stats)
    torch.cuda.synchronize()
    f.check_errors()
    assert np.all(np.isfinite(stats.cpu().numpy()))
    return f, gt


def _eval_kl(synth, f, gt):
    import torch
    rng = np.random.default_rng(EVAL_SEED + 7)
    q = synth.wavefront(N_EVAL, seed=EVAL_SEED)
    cell = gt.cell(q["pos"].astype(np.float64))
    wi = gt.sample(rng, cell)
    log_g = np.log(gt.density(cell, wi))
    dev = {k: torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("pos", "wo", "normal", "rough")}
    p = f.pdf(dev["pos"], dev["wo"], dev["normal"], dev["rough"],
              torch.from_numpy(wi.astype(np.float32)).cuda()).cpu().numpy().astype(np.float64)
    kl_guide = float(np.mean(log_g - np.log(np.maximum(p, 1e-30))))
    kl_uniform = float(np.mean(log_g + math.log(4 * math.pi)))
    # the reference's cosine lobe (kappa 2.18853 around the normal) as a proposal without a network
    n = q["normal"].astype(np.float64)
    k = 2.18853
    c = (n * wi).sum(1)
    log_cos = np.log(k / (2 * math.pi * -np.expm1(-2 * k))) + k * (c - 1)
    kl_cos = float(np.mean(log_g - log_cos))
    return kl_guide, kl_uniform, kl_cos


@pytest.fixture(scope="module")
def fp32_run(nmg, synth):
    f, gt = _train(nmg, synth, nmg.PATH_FP32)
    kl = _eval_kl(synth, f, gt)
    f.close()
    return kl


def test_trained_guide_beats_proposals_without_network(nmg, synth, fp32_run):
    f, gt = _train(nmg, synth, nmg.PATH_BF16)
    kl_guide, kl_uniform, kl_cos = _eval_kl(synth, f, gt)
    print(f"KL(g||guide) = {kl_guide:.4f} (FP32 path {fp32_run[0]:.4f}), uniform = {kl_uniform:.4f}, "
          f"cosine lobe = {kl_cos:.4f}")
    assert kl_guide < 0.75 * kl_uniform
    assert kl_guide < 0.5 * kl_cos
    f.close()


@pytest.mark.parametrize("path", ["bf16", "fp16"])
def test_reduced_precision_converges_like_fp32(nmg, synth, fp32_run, path):
    """Same initialisation, data and steps: the fused BF16 (FP16) path's final KL is at most 2% above
    the plain FP32 path's (measured: 3.5% / 1.6% below it), and not implausibly far below."""
    f, gt = _train(nmg, synth, {"bf16": nmg.PATH_BF16, "fp16": nmg.PATH_FP16}[path])
    kl, kl_u, _ = _eval_kl(synth, f, gt)
    kl32 = fp32_run[0]
    print(f"KL fp32 = {kl32:.4f}, {path} = {kl:.4f}, uniform = {kl_u:.4f}")
    assert kl32 < 0.75 * kl_u
    assert kl <= 1.02 * kl32
    assert kl >= 0.90 * kl32
    f.close()


CONFIG2_SEEDS = (7272, 7273, 7274)


def test_config2_settings_lr_1e2_500_steps(nmg, synth):
    """The full-step configuration at its own optimiser settings (Adam at the reference's learning rate
    1e-2, common/configs/nn/base.json, 500 steps of 2^18 fresh records, K = 8), for the FP32, BF16 and
    FP16 paths on three seeds each: the held-out KL of each run, and whether it collapsed to the uniform
    density (KL within 5% of the uniform sphere's)."""
    import torch
    global LR
    rows = []
    saved = LR
    try:
        LR = 1e-2
        for seed in CONFIG2_SEEDS:
            row = {"seed": seed}
            for name, path in (("fp32", nmg.PATH_FP32), ("bf16", nmg.PATH_BF16), ("fp16", nmg.PATH_FP16)):
                f, gt = _train(nmg, synth, path, steps=500, seed=seed)
                kl, kl_u, _ = _eval_kl(synth, f, gt)
                f.close()
                row[name] = kl
                row["uniform"] = kl_u
            rows.append(row)
    finally:
        LR = saved
    print("\nconfig 2 (lr 1e-2, 500 steps): held-out KL(g || guide)")
    print("| seed | FP32 | BF16 | FP16 | uniform sphere |")
    print("|---|---|---|---|---|")
    for r in rows:
        print("| %d | %.4f | %.4f | %.4f | %.4f |" % (r["seed"], r["fp32"], r["bf16"], r["fp16"], r["uniform"]))
    # Every run ends finite and no worse than the uniform density by more than 5% (collapse lands on
    # the uniform density itself: the lobes' kappa at the exp clamp's floor)
    for r in rows:
        for k in ("fp32", "bf16", "fp16"):
            assert np.isfinite(r[k]) and r[k] <= 1.05 * r["uniform"], (r["seed"], k, r[k])
