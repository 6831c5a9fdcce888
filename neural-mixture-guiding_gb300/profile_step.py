"""Run the guiding step a few times on a fixed workload, for profilers (ncu).

    python neural-mixture-guiding_gb300/profile_step.py [--path bf16|fp16|fp32]
        [--queries N] [--train N] [--repeat R] [--mixture N] [--tiling T]

Builds one guiding field (hash-grid network), runs R query passes over an N-query
synthetic wavefront and, with --train, R training steps of that many records.
With --mixture N it runs the mixture-only kernels instead (R x sample, pdf and
loss/gradient on N synthetic raw rows, K = --lobes). --tiling selects the query
kernel's tiling (nmg_set_query_tiling; 0 = the default).
Prints "ok" on success. Nothing is timed here: profile with e.g.
    ncu --set full --clock-control none -k regex:k_fused_query -s 2 -c 1 -o prof \\
        python neural-mixture-guiding_gb300/profile_step.py
"""
import argparse
import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
PKG = "neural-mixture-guiding_gb300"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--path", default="bf16", choices=["bf16", "fp16", "fp32"])
    ap.add_argument("--queries", type=int, default=1920 * 1080)
    ap.add_argument("--train", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--lobes", type=int, default=8)
    ap.add_argument("--mixture", type=int, default=0)
    ap.add_argument("--tiling", type=int, default=0)
    args = ap.parse_args()
    import torch

    nmg = importlib.import_module(PKG)
    synth = importlib.import_module(PKG + ".synth")
    if args.mixture:
        raw, u4, rec = synth.mixture_batch(args.mixture, args.lobes, seed=1)
        wi = synth.uniform_sphere(np.random.default_rng(2), (args.mixture,)).astype(np.float32)
        r, u, rc, w = (torch.from_numpy(a).cuda() for a in (raw, u4, rec, wi))
        for _ in range(args.repeat):
            nmg.mixture_sample(r, u, args.lobes)
            nmg.mixture_pdf(r, w, args.lobes)
            nmg.mixture_loss_grad(r, rc, args.lobes)
        torch.cuda.synchronize()
        print("ok")
        return
    path = {"bf16": nmg.PATH_BF16, "fp16": nmg.PATH_FP16, "fp32": nmg.PATH_FP32}[args.path]
    f = nmg.GuidingField(nmg.config(nmg.PRESET_HASHGRID, path=path, n_lobes=args.lobes),
                         max_queries=args.queries, max_batch=args.train)
    f.set_query_tiling(args.tiling)
    if args.queries:
        q = synth.wavefront(args.queries, seed=1)
        pos, wo, n, r, u4 = (torch.from_numpy(q[k]).cuda() for k in ("pos", "wo", "normal", "rough", "u4"))
        out = None
        for _ in range(args.repeat):
            out = f.query(pos, wo, n, r, u4, outputs=out)
    if args.train:
        gt = synth.TrainField(seed=1)
        x, rec = synth.train_batch(gt, args.train, seed=2, input_mode=1, selection=True)
        xd, rd = torch.from_numpy(x).cuda(), torch.from_numpy(rec).cuda()
        for _ in range(args.repeat):
            f.train_step(xd, rd)
    torch.cuda.synchronize()
    print("ok")


if __name__ == "__main__":
    main()
