"""The fused tensor-core path (tcgen05 MLP, BF16 or FP16 operands, FP32
accumulate) against the FP64 oracle.

  * raw network outputs: compared with the FP64 oracle evaluated on the
    parameter values the kernels multiply (GuidingField.operand_params: the
    16-bit grid table; for the BF16 path's query image W0 as a BF16 hi + lo
    pair and FP16 later layers), so the remaining difference is the rounding
    of encoded features and hidden activations to 16 bits (2^-9 relative for
    BF16, 2^-11 for FP16) accumulated over the layers:
    max |err| <= 4e-2 (BF16) / 1e-2 (FP16) of max |y|, RMS <= 6e-3 / 2e-3 of RMS y.
    A wrong operand layout or descriptor gives O(1) errors.
  * mixture stage (fast-math FP32 on the fused kernel's own raw outputs):
    lobe index as the FP32 path, direction 1e-3, pdf relative 1e-3
    (+ 4e-7 kappa_max conditioning).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def round16(x, fp16):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32))
    return t.to(torch.float16 if fp16 else torch.bfloat16).to(torch.float32).numpy()


CASES = [(1, 1, 8), (1, 2, 8), (0, 1, 8), (1, 1, 16)]  # (preset, path, K)


@pytest.fixture(params=CASES, ids=["hash-bf16", "hash-fp16", "reference-bf16", "hash-bf16-K16"])
def field(request, nmg, oracle):
    preset, path, K = request.param
    cfg = nmg.config(preset, path=path, n_lobes=K)
    f = nmg.GuidingField(cfg, max_queries=16384, max_batch=4096)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    yield f, net, path == 2
    f.close()


def perturb(f, seed):
    """Replace the (tiny) initial grid table by O(0.1) values so that the grid features matter."""
    import torch
    p = f.get_params(0)
    g = torch.Generator(device="cuda").manual_seed(seed)
    n_mlp = int(f.info.n_mlp_params)
    p[n_mlp:] = 0.2 * torch.randn(p.numel() - n_mlp, device="cuda", generator=g)
    f.set_params(p)


def test_fused_raw_outputs(field, oracle, synth):
    f, net, fp16 = field
    perturb(f, 1)
    q = synth.wavefront(16384, seed=11)
    x = synth.featurize(q, f.cfg.input_mode)
    raw = f.infer_raw(dev(x)[0], which=1).cpu().numpy()
    w16 = f.operand_params(1).cpu().numpy()
    raw64 = oracle.network_forward(net, w16, x)
    nu = net.n_out_padded
    err = np.abs(raw[:, :nu] - raw64[:, :nu])
    scale_max = np.abs(raw64).max()
    rms = np.sqrt((raw64 ** 2).mean())
    assert err.max() <= (1e-2 if fp16 else 4e-2) * scale_max, (err.max(), scale_max)
    assert np.sqrt((err ** 2).mean()) <= (2e-3 if fp16 else 6e-3) * rms, (np.sqrt((err ** 2).mean()), rms)


def test_fused_query_mixture(field, oracle, synth):
    f, net, fp16 = field
    perturb(f, 2)
    K = f.cfg.n_lobes
    q = synth.wavefront(16384, seed=12)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    out = f.query(pos, wo, n, r, u4, want_raw=True)
    raw = out["raw"].cpu().numpy()
    # the raw outputs of the query agree with infer_raw on nmg_featurize's rows; the query featurises
    # with a precomputed box and rsqrt, so the inputs differ by ulps, which the 16-bit rounding of the
    # encoded features can turn into one operand ulp
    x = f.featurize(pos, wo, n, r)
    raw2 = f.infer_raw(x, which=1).cpu().numpy()
    assert np.abs(raw - raw2).max() <= 2e-2 * max(1.0, np.abs(raw2).max())
    assert np.sqrt(((raw - raw2) ** 2).mean()) <= 2e-4 * max(1.0, np.abs(raw2).max())
    s = np.where((q["normal"] * q["wo"]).sum(1, keepdims=True) > 0, 1.0, -1.0).astype(np.float32)
    cosn = (q["normal"] * s).astype(np.float32)
    d64, _, lb64 = oracle.mixture_sample(raw, K, q["u4"], cosn, fp64=True)
    bd = oracle.boundary_distance(raw, K, q["u4"], cosn)
    lb = out["lobe"].cpu().numpy()
    assert np.all((lb == lb64) | (bd < 1e-5))
    ok = lb == lb64
    d = out["dir"].cpu().numpy()
    assert np.abs(d[ok] - d64[ok]).max() <= 1e-3
    p64 = oracle.mixture_pdf(raw, K, d, cosn, fp64=True)
    kmax = np.exp(np.clip(raw[:, 1:4 * K:4].astype(np.float64), -10, 15)).max(axis=1) + 2.2
    rel = np.abs(out["pdf"].cpu().numpy() - p64) / p64
    assert np.all(rel <= 1e-3 + 4e-7 * kmax), rel.max()
    if f.cfg.selection:
        sel = out["selection"].cpu().numpy()
        assert np.abs(sel - 1 / (1 + np.exp(-raw[:, 4 * K].astype(np.float64)))).max() < 1e-4


def test_fused_query_without_raw_matches_query_with_raw(field, synth):
    """A query that returns no raw outputs (for 16 lobes: the epilogue that re-reads each lobe group
    from TMEM instead of holding all raw outputs in registers) returns what the raw-returning query
    returns: the same lobes, directions and pdfs up to FMA-contraction ulps."""
    f, _, _ = field
    perturb(f, 3)
    q = synth.wavefront(16384, seed=16)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    a = f.query(pos, wo, n, r, u4, want_raw=True)
    b = f.query(pos, wo, n, r, u4)
    same = a["lobe"] == b["lobe"]
    assert float(same.float().mean()) >= 0.9999
    assert float((a["dir"] - b["dir"])[same].abs().max()) <= 1e-5
    assert float(((a["pdf"] - b["pdf"]).abs() / a["pdf"])[same].max()) <= 1e-5
    if f.cfg.selection:
        assert float((a["selection"] - b["selection"]).abs().max()) <= 1e-6
    f.check_errors()


def test_fused_pdf_at_given_directions(field, oracle, synth):
    """nmg_pdf in one fused pass: at the query's own sampled directions it returns the query's pdf, and at
    arbitrary directions it matches the FP64 mixture on the network's raw outputs; rows past the device
    count stay untouched."""
    import torch
    f, net, fp16 = field
    perturb(f, 4)
    K = f.cfg.n_lobes
    q = synth.wavefront(16384, seed=14)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    out = f.query(pos, wo, n, r, u4, want_raw=True)
    p_own = f.pdf(pos, wo, n, r, out["dir"])
    rel = ((p_own - out["pdf"]).abs() / out["pdf"]).max().item()
    assert rel <= 1e-6, rel
    wi = synth.uniform_sphere(np.random.default_rng(15), (16384,)).astype(np.float32)
    p = f.pdf(pos, wo, n, r, dev(wi)[0]).cpu().numpy()
    raw = out["raw"].cpu().numpy()
    s = np.where((q["normal"] * q["wo"]).sum(1, keepdims=True) > 0, 1.0, -1.0).astype(np.float32)
    p64 = oracle.mixture_pdf(raw, K, wi, (q["normal"] * s).astype(np.float32), fp64=True)
    kmax = np.exp(np.clip(raw[:, 1:4 * K:4].astype(np.float64), -10, 15)).max(axis=1) + 2.2
    assert np.all(np.abs(p - p64) / p64 <= 1e-3 + 4e-7 * kmax)
    cnt = torch.tensor([5000], dtype=torch.int32, device="cuda")
    pc = torch.full((16384,), -1.0, device="cuda")
    wid = dev(wi)[0]
    st = f.L.nmg_pdf(f.h, ctypes.byref(f.shading(pos, wo, n, r)), wid.data_ptr(), cnt.data_ptr(), 16384,
                     pc.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    assert torch.equal(pc[:5000].cpu(), torch.from_numpy(p[:5000])) and bool((pc[5000:] == -1.0).all())
    f.check_errors()


def test_fused_device_count_and_ragged(field, synth):
    import torch
    f, _, _ = field
    q = synth.wavefront(1000, seed=13)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    full = f.query(pos, wo, n, r, u4)
    for c in (0, 1, 127, 128, 129, 613, 1000):
        cnt = torch.tensor([c], dtype=torch.int32, device="cuda")
        out = {"dir": torch.full((1000, 3), 7.0, device="cuda"), "pdf": torch.full((1000,), -1.0, device="cuda"),
               "lobe": torch.full((1000,), -5, dtype=torch.int32, device="cuda")}
        f.query(pos, wo, n, r, u4, count=cnt, outputs=out)
        assert torch.equal(out["pdf"][:c], full["pdf"][:c]) and torch.equal(out["lobe"][:c], full["lobe"][:c])
        assert bool((out["pdf"][c:] == -1).all())
    f.L.nmg_check_errors.argtypes = [__import__("ctypes").c_void_p]
    assert f.L.nmg_check_errors(f.h) == 0


def block_errors(g, g64, net):
    offs = [0]
    w_in = net.n_enc_padded
    for _ in range(net.n_hidden):
        offs.append(offs[-1] + net.width * w_in)
        w_in = net.width
    offs.append(offs[-1] + net.n_out_padded * net.width)
    offs.append(net.n_params)
    out = []
    for a, b in zip(offs[:-1], offs[1:]):
        ref, got = g64[a:b], g[a:b]
        out.append((np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-30),
                    np.sqrt(((got - ref) ** 2).mean()) / max(np.sqrt((ref ** 2).mean()), 1e-30)))
    return out


def split_mlp(net, w):
    """Weight matrices (row-major [out][in]) of a parameter vector."""
    mats, off, w_in = [], 0, net.n_enc_padded
    for _ in range(net.n_hidden):
        mats.append(w[off:off + net.width * w_in].reshape(net.width, w_in))
        off += net.width * w_in
        w_in = net.width
    mats.append(w[off:off + net.n_out_padded * net.width].reshape(net.n_out_padded, net.width))
    return mats


def emulate_fused_gradient(oracle, net, w16, x, rec, K, sel, fp16):
    """The fused training kernel's arithmetic on the host: FP64 products with 16-bit rounding exactly
    where the kernel stores a 16-bit operand tile (encoded inputs, hidden activations, deltas), the
    adjoint from the FP64 oracle, and the delta range factor S (n for BF16, min(n, 256) for FP16)."""
    import torch
    dt = torch.float16 if fp16 else torch.bfloat16

    def rnd(t):
        return t.to(dt).to(torch.float64)

    n = x.shape[0]
    S = float(min(n, 256) if fp16 else n)
    _, enc = oracle.network_forward(net, w16, x, want_enc=True)
    W = [torch.from_numpy(m.astype(np.float64)) for m in split_mlp(net, w16)]
    a0 = rnd(torch.from_numpy(enc))
    h0 = rnd(torch.relu(a0 @ W[0].T))
    h1 = rnd(torch.relu(h0 @ W[1].T))
    h2 = rnd(torch.relu(h1 @ W[2].T))
    raw = (h2 @ W[3].T).numpy()
    g, _, tot = oracle.mixture_loss_grad(raw.astype(np.float32), K, rec, 128.0, selection=sel, fp64=True)
    d3 = rnd(torch.from_numpy(g) * S)
    dW3 = d3.T @ h2
    d2 = rnd((d3 @ W[3]) * (h2 > 0))
    dW2 = d2.T @ h1
    d1 = rnd((d2 @ W[2]) * (h1 > 0))
    dW1 = d1.T @ h0
    d0 = rnd((d1 @ W[1]) * (h0 > 0))
    dW0 = d0.T @ a0
    denc = (d0 @ W[0]).numpy()
    grid = oracle.grid_backward(net, x, denc)
    mlp = np.concatenate([m.numpy().ravel() for m in (dW0, dW1, dW2, dW3)])
    return np.concatenate([mlp, grid]) / S, tot


@pytest.mark.parametrize("n", [4096, 40000], ids=["one-tile-per-cta", "multi-tile"])
def test_fused_train_gradient(field, oracle, synth, n):
    """One fused training step: the loss-scaled gradient against the host emulation of the same 16-bit
    rounding points (tight), and against the FP64 oracle on the same 16-bit weights (loose, the
    precision cost of 16-bit activations). 40,000 records give every CTA more than one tile, so the
    TMEM weight-gradient accumulation across tiles is exercised."""
    f, net, fp16 = field
    perturb(f, 3)
    K, sel = f.cfg.n_lobes, bool(f.cfg.selection)
    f.reserve(0, n)
    gt = synth.TrainField(seed=5)
    x, rec = synth.train_batch(gt, n, seed=6, input_mode=f.cfg.input_mode, selection=sel)
    w16 = round16(f.get_params(0).cpu().numpy(), fp16)
    stats = f.train_step(*dev(x, rec)).cpu().numpy()
    g = f.get_gradients().cpu().numpy()
    g_emu, tot = emulate_fused_gradient(oracle, net, w16, x, rec, K, sel, fp16)
    errs = block_errors(g, g_emu, net)
    for i, (emax, erms) in enumerate(errs):
        assert erms <= 5e-3 and emax <= 5e-2, ("emulation", i, emax, erms)
    raw64 = oracle.network_forward(net, w16, x)
    graw, _, tot64 = oracle.mixture_loss_grad(raw64.astype(np.float32), K, rec, 128.0, selection=sel, fp64=True)
    g64 = oracle.network_backward(net, w16, x, graw)
    for i, (emax, erms) in enumerate(block_errors(g, g64, net)):
        assert erms <= (0.02 if fp16 else 0.10), ("fp64", i, emax, erms)
    assert abs(stats[0] - tot64 / n) <= 2e-2 * abs(tot64 / n)
    assert f.step == 1
    f.L.nmg_check_errors.argtypes = [__import__("ctypes").c_void_p]
    assert f.L.nmg_check_errors(f.h) == 0


def test_fused_train_large_batch_and_ragged(field, synth):
    """Batches that are not a multiple of the 128-row tile and larger than one tile per SM run
    without error, and the device count clamps the batch."""
    import torch
    f, net, fp16 = field
    gt = synth.TrainField(seed=7)
    x, rec = synth.train_batch(gt, 4000, seed=8, input_mode=f.cfg.input_mode, selection=bool(f.cfg.selection))
    xd, rd = dev(x, rec)
    s1 = f.train_step(xd, rd).cpu().numpy()
    cnt = torch.tensor([1234], dtype=torch.int32, device="cuda")
    s2 = f.train_step(xd, rd, count=cnt).cpu().numpy()
    assert np.all(np.isfinite(s1)) and np.all(np.isfinite(s2))
    f.L.nmg_check_errors.argtypes = [__import__("ctypes").c_void_p]
    assert f.L.nmg_check_errors(f.h) == 0


@pytest.mark.parametrize("preset,path,K", [(1, 1, 8), (0, 1, 8), (1, 1, 16)], ids=["hash-bf16", "reference-bf16", "hash-K16"])
def test_fused_train_many_tiles_per_group(nmg, synth, preset, path, K):
    """2^18 records: every compute warpgroup walks ~7 tiles, so the hand-offs between tiles (the
    grid-gradient staging read by the scatter warps while the group encodes its next tile) are
    exercised many times. Two identically initialised fields give the same gradient up to the order
    of the float atomics, and the gradient agrees with the plain FP32 path's at the BF16 budget."""
    import torch
    n = 1 << 18
    gt = synth.TrainField(seed=21)
    cfg = nmg.config(preset, path=path, n_lobes=K)
    x, rec = synth.train_batch(gt, n, seed=22, input_mode=cfg.input_mode, selection=bool(cfg.selection))
    xd, rd = dev(x, rec)
    grads = []
    for _ in range(2):
        f = nmg.GuidingField(cfg, max_batch=n)
        perturb(f, 23)
        f.train_step(xd, rd)
        grads.append(f.get_gradients())
        f.check_errors()
        f.close()
    g1, g2 = grads
    scale = float(g1.abs().max())
    assert float((g1 - g2).abs().max()) <= 1e-4 * scale
    f32 = nmg.GuidingField(nmg.config(preset, path=nmg.PATH_FP32, n_lobes=K), max_batch=n)
    perturb(f32, 23)
    f32.train_step(xd, rd)
    g32 = f32.get_gradients()
    f32.close()
    rel = float((g1 - g32).pow(2).sum().sqrt() / g32.pow(2).sum().sqrt())
    assert rel <= 0.1, rel


def test_fused_tilings_agree_and_autotune(nmg, synth, tmp_path, monkeypatch):
    """Every CTA tiling of the fused query kernel computes the same outputs up to instruction-level
    contraction (each tiling is its own compiled instantiation, and the assembler may fuse a multiply
    and an add in one and not in another, which can move a BF16 hidden activation by one ulp): raw
    outputs within the BF16 budget, almost every sample in the same lobe with the same direction. The autotuner picks one
    tiling and caches it."""
    import torch
    monkeypatch.setenv("NMG_TUNE_CACHE", str(tmp_path / "tune.txt"))
    f = nmg.GuidingField(nmg.config(1, path=1), max_queries=50000)
    q = synth.wavefront(50000, seed=21)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    ref = None
    ran = []
    for wg in (4, 5, 6, 8, 9, 10, 11, 12):
        f.set_query_tiling(wg)
        try:
            out = f.query(pos, wo, n, r, u4, want_raw=True)
        except nmg.NMGError as e:
            # a tiling whose shared memory does not fit this network's weight image (the 8-slot ring
            # with the BF16 path's extra layer-0 image) reports UNSUPPORTED and is skipped
            assert e.status == 6, e
            continue
        ran.append(wg)
        if ref is None:
            ref = out
        else:
            raw_err = (out["raw"] - ref["raw"]).abs() / ref["raw"].abs().clamp(min=1.0)
            assert float(raw_err.max()) <= 2e-2, wg
            assert float(raw_err.pow(2).mean().sqrt()) <= 2e-4, wg
            same = out["lobe"] == ref["lobe"]
            assert float(same.float().mean()) >= 0.999, wg
            assert float((out["dir"] - ref["dir"])[same].abs().max()) <= 5e-2, wg
            assert float(((out["dir"] - ref["dir"])[same]).pow(2).mean().sqrt()) <= 1e-3, wg
            rel = (out["pdf"] - ref["pdf"])[same].abs() / ref["pdf"][same]
            assert float(rel.pow(2).mean().sqrt()) <= 1e-3, wg
    assert len(ran) >= 6 and 12 in ran and 4 in ran
    chosen = f.autotune(pos, wo, n, r, u4, use_cache=True)
    assert chosen in ran and f.query_tiling == chosen
    assert (tmp_path / "tune.txt").read_text().strip().endswith(str(chosen))
    f.set_query_tiling(0)
    assert f.autotune(pos, wo, n, r, u4, use_cache=True) == chosen  # served from the cache
    f.check_errors()
    f.close()


@pytest.mark.parametrize("preset,K", [(1, 8), (1, 16), (0, 8)], ids=["hash-K8", "hash-K16", "reference-K8"])
def test_pair_tiling_matches_one_thread_per_query(nmg, synth, preset, K):
    """Tiling 7 (two threads per query, the lobes split between them, the selection scan continued by
    the second thread) samples the same lobes and directions and evaluates the same pdfs as tiling 4 (one
    thread per query) on the same inputs, up to the order of the lobe sums and instruction-level
    contraction: sampling, and the pdf at given directions."""
    f = nmg.GuidingField(nmg.config(preset, path=1, n_lobes=K), max_queries=50000)
    perturb(f, 7)
    q = synth.wavefront(50000, seed=23)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    f.set_query_tiling(4)
    ref = f.query(pos, wo, n, r, u4)
    pref = f.pdf(pos, wo, n, r, ref["dir"])
    f.set_query_tiling(7)
    out = f.query(pos, wo, n, r, u4)
    pout = f.pdf(pos, wo, n, r, ref["dir"])
    same = out["lobe"] == ref["lobe"]
    assert float(same.float().mean()) >= 0.999
    assert float((out["dir"] - ref["dir"])[same].abs().max()) <= 5e-2
    assert float(((out["dir"] - ref["dir"])[same]).pow(2).mean().sqrt()) <= 1e-3
    rel = (out["pdf"] - ref["pdf"])[same].abs() / ref["pdf"][same]
    assert float(rel.pow(2).mean().sqrt()) <= 1e-3
    relp = (pout - pref).abs() / pref
    assert float(relp.pow(2).mean().sqrt()) <= 1e-3
    if "selection" in ref:
        assert float((out["selection"] - ref["selection"]).abs().max()) <= 1e-3
    f.check_errors()
    f.close()


@pytest.mark.parametrize("tiling", [7, 8, 4])
def test_16_lobe_direction_stores_any_alignment(nmg, synth, tiling):
    """The 16-lobe epilogues write a warp's 32 directions as whole-sector float4 rows when the
    output is 16-byte aligned and every row of the warp is valid, and row by row otherwise. A
    direction array starting 12 bytes into an allocation (not 16-byte aligned) and a ragged
    count (a partial last warp) give the same outputs as an aligned array."""
    import torch
    n = 40_007
    f = nmg.GuidingField(nmg.config(1, path=1, n_lobes=16), max_queries=n)
    perturb(f, 11)
    f.set_query_tiling(tiling)
    q = synth.wavefront(n, seed=31)
    pos, wo, nrm, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    ref = f.query(pos, wo, nrm, r, u4)
    back = torch.full((n + 1, 3), float("nan"), device="cuda")
    out = {"dir": back[1:], "pdf": torch.empty(n, device="cuda"),
           "lobe": torch.empty(n, device="cuda", dtype=torch.int32)}
    assert out["dir"].data_ptr() % 16 == 12
    f.query(pos, wo, nrm, r, u4, outputs=out)
    torch.cuda.synchronize()
    assert torch.equal(out["dir"], ref["dir"])
    assert torch.equal(out["pdf"], ref["pdf"])
    assert torch.isnan(back[0]).all()  # nothing written before the array
    f.check_errors()
    f.close()
