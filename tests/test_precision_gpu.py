"""Error of every output of the guiding step against the FP64 oracle, per
precision path (the precision configuration: 65,536 queries, K = 8, and a
16,384-record training step on the hash-grid network), with the tolerances
each path must meet.

Each path builds the hash-grid guiding field (16x2 hash grid, SH-4 x2,
one-blob 4, 80-64-64-64-48 MLP, K = 8 + selection) from the same seed and
replaces the initial grid table by the same O(0.1) values so that the grid
features matter. The oracle evaluates the FP64 network on the FP32 weights
(the master copy, whose inference copy the query reads), so the 16-bit
paths' errors include the rounding of their parameters. Outputs:
  * raw network outputs (max error relative to max |y|, RMS relative to RMS y);
  * the sampled lobe (equal to the FP64 mixture's choice under the same
    uniforms), the sampled direction where the lobes agree, and the pdf at
    the path's own direction against the FP64 mixture of the FP64 network's
    outputs (end to end) and of the path's own outputs (mixture arithmetic);
  * one training step: mean loss and the parameter gradient (RMS error
    relative to the RMS gradient: all parameters, the grid table, the last
    matrix);
  * the mixture-only FP32 kernels on raw outputs (65,536 queries, K = 8).

Tolerances:
  * plain FP32 path: lobe index equal except uniforms within 1e-6 of an FP64
    CDF boundary; direction 1e-4; pdf 1e-4 + 4e-7 kappa_max relative (an FP32
    direction is known to ~6e-8, which exp(kappa (cos - 1)) amplifies by
    kappa); raw outputs 1e-4 of max |y|; gradients 1e-3 (RMS relative);
  * BF16 and FP16 fused paths: pdf at the sampled direction 1e-3 relative
    at the maximum; the mixture arithmetic on the path's own raw outputs
    1e-5; mean loss 1e-3;
  * mixture-only FP32 kernels: lobe index as above, direction 1e-4, pdf
    1e-4 + 4e-7 kappa_max, loss sum 1e-6, gradient 1e-3 of each row's
    largest component (at least 1).
The last test prints the table of measured errors (pytest -s shows it)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NQ, NB = 65536, 16384
RESULTS = {}


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


def kappa_max(raw, K):
    return np.exp(np.clip(raw[:, 1:4 * K:4].astype(np.float64), -10, 15)).max(axis=1)


def run_path(nmg, synth, O, path):
    import torch
    cfg = nmg.config(nmg.PRESET_HASHGRID, path=path)
    K, sel = int(cfg.n_lobes), bool(cfg.selection)
    f = nmg.GuidingField(cfg, max_queries=NQ, max_batch=NB)
    try:
        p = f.get_params(0)
        n_mlp = int(f.info.n_mlp_params)
        g = torch.Generator(device="cuda").manual_seed(1)
        p[n_mlp:] = 0.2 * torch.randn(p.numel() - n_mlp, device="cuda", generator=g)
        f.set_params(p)
        net = O.make_net(**nmg.oracle_net_spec(cfg))
        w32 = f.get_params(1).cpu().numpy()
        q = synth.wavefront(NQ, seed=12)
        dq = [torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("pos", "wo", "normal", "rough", "u4")]
        out = f.query(*dq, want_raw=True)
        raw = out["raw"].cpu().numpy()
        x = f.featurize(*dq[:4]).cpu().numpy()
        nu = net.n_out_padded
        raw64 = O.network_forward(net, w32, x)
        res = {"raw": scaled_err(raw[:, :nu], raw64[:, :nu])}
        s = np.where((q["normal"] * q["wo"]).sum(1, keepdims=True) > 0, 1.0, -1.0).astype(np.float32)
        cosn = (q["normal"] * s).astype(np.float32)
        r64f = raw64.astype(np.float32)
        d64, _, lb64 = O.mixture_sample(r64f, K, q["u4"], cosn, fp64=True)
        bd = O.boundary_distance(r64f, K, q["u4"], cosn)
        lb, d, pdf = out["lobe"].cpu().numpy(), out["dir"].cpu().numpy(), out["pdf"].cpu().numpy()
        same = lb == lb64
        res["lobe_equal_fraction"] = float(same.mean())
        res["lobe_mismatch_off_boundary"] = int((~same & (bd > 1e-6)).sum())
        res["direction_abs_err"] = abs_stats(np.abs(d[same] - d64[same]).max(axis=1))
        p64 = O.mixture_pdf(r64f, K, d, cosn, fp64=True)
        res["pdf_end_to_end"] = rel_stats(pdf, p64)
        res["pdf_end_to_end_rel"] = np.abs(pdf - p64) / p64
        res["kappa_max"] = kappa_max(r64f, K) + 2.2  # the cosine lobe's kappa bounds the product's increase
        res["pdf_mixture_only"] = rel_stats(pdf, O.mixture_pdf(raw, K, d, cosn, fp64=True))
        gt = synth.TrainField(seed=5)
        xt, rec = synth.train_batch(gt, NB, seed=6, input_mode=cfg.input_mode, selection=sel)
        wm = f.get_params(0).cpu().numpy()
        stats = f.train_step(torch.from_numpy(xt).cuda(), torch.from_numpy(rec).cuda()).cpu().numpy()
        grad = f.get_gradients().cpu().numpy()
        t64 = O.network_forward(net, wm, xt)
        graw, _, tot64 = O.mixture_loss_grad(t64.astype(np.float32), K, rec, 128.0, selection=sel, fp64=True)
        g64 = O.network_backward(net, wm, xt, graw)
        res["train_mean_loss_rel_err"] = float(abs(stats[0] - tot64 / NB) / abs(tot64 / NB))
        res["gradient"] = {name: scaled_err(grad[a:b], g64[a:b])["rms_rel_to_rms"] for name, a, b in blocks(net)}
        res["gradient"]["all"] = scaled_err(grad, g64)["rms_rel_to_rms"]
        f.check_errors()
        return res
    finally:
        f.close()


@pytest.fixture(scope="module")
def path_result(request, nmg, synth, oracle):
    def get(name):
        if name not in RESULTS:
            path = {"fp32": nmg.PATH_FP32, "bf16": nmg.PATH_BF16, "fp16": nmg.PATH_FP16}[name]
            RESULTS[name] = run_path(nmg, synth, oracle, path)
        return RESULTS[name]
    return get


def test_fp32_plain_path(path_result):
    r = path_result("fp32")
    assert r["raw"]["max_rel_to_max"] <= 1e-4
    assert r["lobe_mismatch_off_boundary"] == 0
    assert r["direction_abs_err"]["max"] <= 1e-4
    assert np.all(r["pdf_end_to_end_rel"] <= 1e-4 + 4e-7 * r["kappa_max"])
    assert r["train_mean_loss_rel_err"] <= 1e-5
    for k in ("all", "grid", "W3"):
        assert r["gradient"][k] <= 1e-3, (k, r["gradient"][k])


@pytest.mark.parametrize("name", ["bf16", "fp16"])
def test_fused_path_pdf_within_1e3(path_result, name):
    r = path_result(name)
    assert r["pdf_end_to_end"]["max"] <= 1e-3, r["pdf_end_to_end"]
    assert r["pdf_mixture_only"]["max"] <= 1e-5, r["pdf_mixture_only"]
    assert r["train_mean_loss_rel_err"] <= 1e-3


def test_mixture_only_fp32_kernels(nmg, synth, oracle):
    import torch
    n, K = NQ, 8
    raw, u4, rec = synth.mixture_batch(n, K, seed=7272)
    r, u, rc = (torch.from_numpy(a).cuda() for a in (raw, u4, rec))
    d, p, lb = nmg.mixture_sample(r, u, K)
    g, loss, tot = nmg.mixture_loss_grad(r, rc, K)
    d, p, lb = d.cpu().numpy(), p.cpu().numpy(), lb.cpu().numpy()
    d64, _, lb64 = oracle.mixture_sample(raw, K, u4, fp64=True)
    bd = oracle.boundary_distance(raw, K, u4)
    same = lb == lb64
    assert not (~same & (bd > 1e-6)).any()
    assert np.abs(d[same] - d64[same]).max() <= 1e-4
    p64 = oracle.mixture_pdf(raw, K, d, fp64=True)
    rel = np.abs(p - p64) / p64
    assert np.all(rel <= 1e-4 + 4e-7 * kappa_max(raw, K))
    g64, _, t64 = oracle.mixture_loss_grad(raw, K, rec, fp64=True)
    assert abs(float(tot.cpu()[0]) - t64) <= 1e-6 * abs(t64)
    gg = g.cpu().numpy()[:, :4 * K]
    rowmax = np.maximum(1.0, np.abs(g64[:, :4 * K]).max(axis=1, keepdims=True))
    assert (np.abs(gg - g64[:, :4 * K]) / rowmax).max() <= 1e-3
    RESULTS["mixture_only"] = {"direction_max": float(np.abs(d[same] - d64[same]).max()),
                               "pdf": rel_stats(p, p64)}


def test_print_precision_table(path_result):
    """The measured errors of every output (the figures the design notes quote)."""
    P = ("fp32", "bf16", "fp16")
    rep = {p: path_result(p) for p in P}
    rows = [("raw outputs, max / RMS (of max, RMS y)",
             lambda r: "%.1e / %.1e" % (r["raw"]["max_rel_to_max"], r["raw"]["rms_rel_to_rms"])),
            ("lobe index equal", lambda r: "%.5f" % r["lobe_equal_fraction"]),
            ("direction (same lobe), median / p99 / max abs", lambda r: "%.1e / %.1e / %.1e" % tuple(
                r["direction_abs_err"][k] for k in ("median", "p99", "max"))),
            ("pdf end to end, median / p99 / max rel", lambda r: "%.1e / %.1e / %.1e" % tuple(
                r["pdf_end_to_end"][k] for k in ("median", "p99", "max"))),
            ("pdf, mixture stage only, max rel", lambda r: "%.1e" % r["pdf_mixture_only"]["max"]),
            ("training mean loss, rel", lambda r: "%.1e" % r["train_mean_loss_rel_err"]),
            ("gradient, RMS rel (all / grid / last matrix)", lambda r: "%.1e / %.1e / %.1e" % (
                r["gradient"]["all"], r["gradient"]["grid"], r["gradient"]["W3"]))]
    print("\n| output (vs FP64 oracle), %d queries, %d records | FP32 plain | BF16 fused | FP16 fused |" % (NQ, NB))
    print("|---|---|---|---|")
    for label, fn in rows:
        print("| %s | %s |" % (label, " | ".join(fn(rep[p]) for p in P)))
    if "mixture_only" in RESULTS:
        m = RESULTS["mixture_only"]
        print("mixture-only FP32 kernels: direction max %.1e, pdf median / p99 / max %.1e / %.1e / %.1e"
              % (m["direction_max"], m["pdf"]["median"], m["pdf"]["p99"], m["pdf"]["max"]))
