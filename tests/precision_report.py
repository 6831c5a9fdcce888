"""Error of every output of the guiding step against the FP64 oracle, per precision path.

    python tests/precision_report.py [--queries N] [--batch B] [--out report.json]

Needs a CUDA device. Builds the hash-grid guiding field (16x2 hash grid, SH-4 x2, one-blob 4,
80-64-64-64-48 MLP, K = 8 + selection) once per path -- plain FP32, fused BF16, fused FP16 --
from the same seed, replaces the initial grid table by O(0.1) values (the same for all three) so
that the grid features matter, and compares with the FP64 oracle evaluated on the FP32 master
weights:
  * raw network outputs of a query pass (max and RMS error relative to max |y| and RMS y), and,
    as a breakdown, against the FP64 network on the path's own 16-bit-rounded weights;
  * lobe index (fraction equal to the FP64 mixture's choice under the same uniforms), sampled
    direction (|d - d64|_inf where the lobes agree: median, 99th percentile, max) and pdf at
    the sampled direction (relative error, max / 99th percentile / median), the oracle's
    mixture fed with the FP64 raw outputs
    (end to end: network + mixture precision) and with the path's own raw outputs (the mixture
    arithmetic alone);
  * one training step: mean loss (relative error) and the parameter gradient (RMS error
    relative to the RMS gradient, per MLP matrix and for the grid table).
Also the mixture-only FP32 kernels on raw outputs (65,536 queries, K = 8): direction, pdf,
loss and gradient error. Prints a markdown table; --out writes the same figures as JSON.
The oracle here is the checker; the measured outputs all come from the CUDA kernels.
"""
import argparse
import importlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
PKG = "neural-mixture-guiding_gb300"


def rel_stats(got, ref):
    r = np.abs(got.astype(np.float64) - ref) / np.abs(ref)
    return {"max": float(r.max()), "p99": float(np.percentile(r, 99)), "median": float(np.median(r))}


def abs_stats(err):
    return {"max": float(err.max()), "p99": float(np.percentile(err, 99)), "median": float(np.median(err))}


def scaled_err(got, ref):
    e = got.astype(np.float64) - ref
    return {"max_rel_to_max": float(np.abs(e).max() / np.abs(ref).max()),
            "rms_rel_to_rms": float(np.sqrt((e ** 2).mean()) / np.sqrt((ref ** 2).mean()))}


def blocks(net):
    offs, w_in = [0], net.n_enc_padded
    for _ in range(net.n_hidden):
        offs.append(offs[-1] + net.width * w_in)
        w_in = net.width
    offs.append(offs[-1] + net.n_out_padded * net.width)
    offs.append(net.n_params)
    names = ["W%d" % i for i in range(net.n_hidden + 1)] + ["grid"]
    return list(zip(names, offs[:-1], offs[1:]))


def network_path(nmg, synth, O, torch, path, nq, nb):
    cfg = nmg.config(nmg.PRESET_HASHGRID, path=path)
    K, sel = int(cfg.n_lobes), bool(cfg.selection)
    f = nmg.GuidingField(cfg, max_queries=nq, max_batch=nb)
    try:
        p = f.get_params(0)
        n_mlp = int(f.info.n_mlp_params)
        g = torch.Generator(device="cuda").manual_seed(1)
        p[n_mlp:] = 0.2 * torch.randn(p.numel() - n_mlp, device="cuda", generator=g)
        f.set_params(p)
        net = O.make_net(**nmg.oracle_net_spec(cfg))
        w32 = f.get_params(1).cpu().numpy()  # the weights the query reads (inference copy), FP32
        dt = {nmg.PATH_BF16: torch.bfloat16, nmg.PATH_FP16: torch.float16}.get(path)
        w16 = torch.from_numpy(w32).to(dt).float().numpy() if dt is not None else w32

        q = synth.wavefront(nq, seed=12)
        dq = [torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("pos", "wo", "normal", "rough", "u4")]
        out = f.query(*dq, want_raw=True)
        raw = out["raw"].cpu().numpy()
        x = f.featurize(*dq[:4]).cpu().numpy()
        nu = net.n_out_padded
        raw64 = O.network_forward(net, w32, x)
        res = {"raw": scaled_err(raw[:, :nu], raw64[:, :nu])}
        if dt is not None:
            res["raw_same_16bit_weights"] = scaled_err(raw[:, :nu], O.network_forward(net, w16, x)[:, :nu])
        s = np.where((q["normal"] * q["wo"]).sum(1, keepdims=True) > 0, 1.0, -1.0).astype(np.float32)
        cosn = (q["normal"] * s).astype(np.float32)
        r64f = raw64.astype(np.float32)
        d64, _, lb64 = O.mixture_sample(r64f, K, q["u4"], cosn, fp64=True)
        lb, d, pdf = out["lobe"].cpu().numpy(), out["dir"].cpu().numpy(), out["pdf"].cpu().numpy()
        same = lb == lb64
        res["lobe_equal_fraction"] = float(same.mean())
        res["direction_abs_err"] = abs_stats(np.abs(d[same] - d64[same]).max(axis=1))
        res["pdf_end_to_end"] = rel_stats(pdf, O.mixture_pdf(r64f, K, d, cosn, fp64=True))
        res["pdf_mixture_only"] = rel_stats(pdf, O.mixture_pdf(raw, K, d, cosn, fp64=True))

        gt = synth.TrainField(seed=5)
        xt, rec = synth.train_batch(gt, nb, seed=6, input_mode=cfg.input_mode, selection=sel)
        wm = f.get_params(0).cpu().numpy()  # FP32 master weights before the step
        stats = f.train_step(torch.from_numpy(xt).cuda(), torch.from_numpy(rec).cuda()).cpu().numpy()
        grad = f.get_gradients().cpu().numpy()
        t64 = O.network_forward(net, wm, xt)
        graw, _, tot64 = O.mixture_loss_grad(t64.astype(np.float32), K, rec, 128.0, selection=sel, fp64=True)
        g64 = O.network_backward(net, wm, xt, graw)
        res["train_mean_loss_rel_err"] = float(abs(stats[0] - tot64 / nb) / abs(tot64 / nb))
        res["gradient"] = {name: scaled_err(grad[a:b], g64[a:b])["rms_rel_to_rms"] for name, a, b in blocks(net)}
        res["gradient"]["all"] = scaled_err(grad, g64)["rms_rel_to_rms"]
        return res
    finally:
        f.close()


def mixture_only(nmg, synth, O, torch, n=65536, K=8):
    raw, u4, rec = synth.mixture_batch(n, K, seed=7272)
    r, u, rc = (torch.from_numpy(a).cuda() for a in (raw, u4, rec))
    d, p, lb = nmg.mixture_sample(r, u, K)
    g, loss, tot = nmg.mixture_loss_grad(r, rc, K)
    d, p, lb = d.cpu().numpy(), p.cpu().numpy(), lb.cpu().numpy()
    d64, _, lb64 = O.mixture_sample(raw, K, u4, fp64=True)
    same = lb == lb64
    g64, l64, t64 = O.mixture_loss_grad(raw, K, rec, fp64=True)
    gg = g.cpu().numpy()[:, :4 * K]
    rowmax = np.maximum(1.0, np.abs(g64[:, :4 * K]).max(axis=1, keepdims=True))
    return {"lobe_equal_fraction": float(same.mean()),
            "direction_abs_err": abs_stats(np.abs(d[same] - d64[same]).max(axis=1)),
            "pdf": rel_stats(p, O.mixture_pdf(raw, K, d, fp64=True)),
            "loss_sum_rel_err": float(abs(float(tot.cpu()[0]) - t64) / abs(t64)),
            "gradient_max_err_rel_to_row_max": float((np.abs(gg - g64[:, :4 * K]) / rowmax).max())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--queries", type=int, default=65536)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    import torch

    import oracle as O
    nmg = importlib.import_module(PKG)
    synth = importlib.import_module(PKG + ".synth")
    rep = {"queries": args.queries, "batch": args.batch, "mixture_only_fp32": mixture_only(nmg, synth, O, torch)}
    for name, path in (("fp32", nmg.PATH_FP32), ("bf16", nmg.PATH_BF16), ("fp16", nmg.PATH_FP16)):
        rep[name] = network_path(nmg, synth, O, torch, path, args.queries, args.batch)
    print(json.dumps(rep, indent=1))
    print()
    print("| output (vs FP64 oracle) | FP32 plain | BF16 fused | FP16 fused |")
    print("|---|---|---|---|")
    P = ("fp32", "bf16", "fp16")
    rows = [("raw outputs, max / RMS (of max, RMS y)",
             lambda r: "%.1e / %.1e" % (r["raw"]["max_rel_to_max"], r["raw"]["rms_rel_to_rms"])),
            ("lobe index equal", lambda r: "%.5f" % r["lobe_equal_fraction"]),
            ("direction (same lobe), median / p99 / max abs", lambda r: "%.1e / %.1e / %.1e" % tuple(
                r["direction_abs_err"][k] for k in ("median", "p99", "max"))),
            ("pdf end to end, median / p99 / max rel", lambda r: "%.1e / %.1e / %.1e" % tuple(
                r["pdf_end_to_end"][k] for k in ("median", "p99", "max"))),
            ("pdf, mixture stage only, max rel", lambda r: "%.1e" % r["pdf_mixture_only"]["max"]),
            ("training mean loss, rel", lambda r: "%.1e" % r["train_mean_loss_rel_err"]),
            ("gradient, RMS rel (all parameters)", lambda r: "%.1e" % r["gradient"]["all"]),
            ("gradient, RMS rel (grid / last matrix)", lambda r: "%.1e / %.1e" % (r["gradient"]["grid"],
                                                                                  r["gradient"]["W3"]))]
    for label, fn in rows:
        print("| %s | %s |" % (label, " | ".join(fn(rep[p]) for p in P)))
    if args.out:
        with open(args.out, "w") as fh:
            json.dump(rep, fh, indent=1)


if __name__ == "__main__":
    main()
