"""Writes tests/golden/mixture_golden.npz from the REFERENCE'S OWN mixture code.

Run in a checkout where the reference exists (it compiles
oracle/_ref/libnmgref.so through oracle/build_ref.sh):

    python tests/golden/make_golden.py

Inputs are seeded synthetic mixtures (neural-mixture-guiding_gb300/synth.py)
plus hand-written edge rows: clamped lambda/kappa logits, lobe means at the
poles, uniforms at 0 and just below 1, directions and normals on the axes.
Outputs come from the reference's distribution.h / vmf.h / train.h compiled
on the host (K = 8, the reference's compile-time lobe count):
  sample  -- MixedSG(raw).sample() + pdf(), with and without applyCosineLobe
  pdf     -- MixedSG(raw).pdf(wi) at given directions
  loss    -- the per-sample body of compute_dL_doutput_divergence
             (train.cu:80-123) with __half raw outputs and gradients.
"""
import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

synth = importlib.import_module("neural-mixture-guiding_gb300.synth")

K = 8
N_RANDOM = 1024
SEED = 7272


def edge_rows(rng):
    rows, u4s = [], []
    base_raw, base_u, _ = synth.mixture_batch(64, K, seed=SEED + 99)
    for i in range(64):
        r = base_raw[i].copy()
        u = base_u[i].copy()
        lobe = i % K
        kind = i // K
        if kind == 0:
            r[4 * lobe + 0] = 20.0   # lambda logit above the exp clamp
        elif kind == 1:
            r[4 * lobe + 0] = -20.0  # below the clamp
            r[4 * lobe + 1] = -20.0  # kappa -> exp(-10)
        elif kind == 2:
            r[4 * lobe + 1] = 9.0    # kappa ~ 8100
        elif kind == 3:
            r[4 * lobe + 2] = 20.0   # theta -> pi (south pole)
            r[4 * lobe + 3] = -20.0  # phi -> 0
        elif kind == 4:
            r[4 * lobe + 2] = -20.0  # theta -> 0 (north pole)
        elif kind == 5:
            u[1] = 0.0
            u[2] = 0.0
        elif kind == 6:
            u[1] = np.float32(0.99999994)
            u[2] = np.float32(0.99999994)
            u[3] = np.float32(0.99999994)
        else:
            r[0:4 * K:4] = 0.0       # equal weights: CDF boundaries at k/8
            u[1] = np.float32(lobe / K)
        rows.append(r)
        u4s.append(u)
    return np.array(rows, np.float32), np.array(u4s, np.float32)


def main():
    if O.ref_lib() is None:
        raise SystemExit("reference checkout not available; cannot regenerate golden vectors")
    rng = np.random.default_rng(SEED)
    raw, u4, rec = synth.mixture_batch(N_RANDOM, K, seed=SEED)
    er, eu = edge_rows(rng)
    raw = np.concatenate([raw, er])
    u4 = np.concatenate([u4, eu])
    n = raw.shape[0]
    _, _, erec = synth.mixture_batch(64, K, seed=SEED + 5)
    rec = np.concatenate([rec, erec])
    axes = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, -1, 0], [-1, 0, 0]], np.float32)
    cosn = synth.uniform_sphere(rng, (n,)).astype(np.float32)
    cosn[:6] = axes
    wi = synth.uniform_sphere(rng, (n,)).astype(np.float32)
    wi[6:12] = axes

    d, p, lb = O.ref_mixture_sample(raw, u4)
    dc, pc, lbc = O.ref_mixture_sample(raw, u4, cosn)
    pe = O.ref_mixture_pdf(raw, wi)
    pec = O.ref_mixture_pdf(raw, wi, cosn)
    g, loss = O.ref_loss_grad(raw, rec, 128.0)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mixture_golden.npz")
    np.savez_compressed(out, K=K, raw=raw, u4=u4, rec=rec, cosn=cosn, wi=wi, dir=d, pdf=p, lobe=lb, dir_cos=dc,
                        pdf_cos=pc, lobe_cos=lbc, pdf_eval=pe, pdf_eval_cos=pec, grad=g, loss=loss,
                        loss_scale=np.float32(128.0))
    print("wrote", out, "rows", n, "bytes", os.path.getsize(out))


if __name__ == "__main__":
    main()
