"""Parity of the network-backed guiding field (nmg_create / nmg_query /
nmg_pdf / nmg_train_step / nmg_network_vjp) with the FP64 oracle.

Paths: the plain FP32 path here; the fused tensor-core paths are covered in
test_fused_gpu.py. Tolerances for the FP32 path:
  * featurised inputs: 2e-6 absolute (values in [0, 1]);
  * raw network outputs: 1e-4 * max(1, |y|) (FP32 accumulation over <=80
    terms per layer);
  * direction / pdf / lobe: as the mixture tests (pdf against the FP64
    oracle evaluated at the GPU's direction on the GPU's raw outputs);
  * parameter gradient: 1e-3 relative to the largest |g| of its block
    (each weight matrix, the grid table);
  * Adam + EMA step: 1e-5 relative on the updated weights.
"""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def face_forward(n, wo):
    s = np.where((n * wo).sum(axis=1, keepdims=True) > 0, 1.0, -1.0).astype(np.float32)
    return (n * s).astype(np.float32)


@pytest.fixture(params=[0, 1], ids=["reference-preset", "hashgrid-preset"])
def field(request, nmg, oracle):
    cfg = nmg.config(request.param, path=nmg.PATH_FP32)
    f = nmg.GuidingField(cfg, max_queries=8192, max_batch=4096)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    yield f, net
    f.close()


def test_featurize(field, oracle, synth):
    f, net = field
    q = synth.wavefront(4096, seed=3)
    # positions partly outside the unit scene box still featurise linearly
    q["pos"] = (q["pos"] * np.float32(1.5) - np.float32(0.25)).astype(np.float32)
    x_or = oracle.featurize(net, q["pos"], q["wo"], q["normal"], q["rough"], q["aabb"])
    pos, wo, n, r = dev(q["pos"], q["wo"], q["normal"], q["rough"])
    x = f.featurize(pos, wo, n, r).cpu().numpy()
    assert x.shape == x_or.shape
    assert np.abs(x - x_or).max() < 2e-6


def test_forward_matches_oracle(field, oracle, synth):
    f, net = field
    q = synth.wavefront(4096, seed=5)
    x = synth.featurize(q, f.cfg.input_mode)
    params = f.get_params(0).cpu().numpy()
    raw = f.infer_raw(dev(x)[0], which=1).cpu().numpy()
    raw64 = oracle.network_forward(net, params, x)
    err = np.abs(raw - raw64).max()
    assert err < 1e-4 * max(1.0, np.abs(raw64).max()), err


def test_query_and_pdf(field, oracle, synth):
    f, net = field
    K = f.cfg.n_lobes
    q = synth.wavefront(8192, seed=6)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    out = f.query(pos, wo, n, r, u4, want_raw=True)
    raw = out["raw"].cpu().numpy()
    x = oracle.featurize(net, q["pos"], q["wo"], q["normal"], q["rough"], q["aabb"])
    raw64 = oracle.network_forward(net, f.get_params(1).cpu().numpy(), x)
    assert np.abs(raw - raw64).max() < 1e-4 * max(1.0, np.abs(raw64).max())
    cosn = face_forward(q["normal"], q["wo"])
    d64, _, lb64 = oracle.mixture_sample(raw, K, q["u4"], cosn, fp64=True)
    bd = oracle.boundary_distance(raw, K, q["u4"], cosn)
    lb = out["lobe"].cpu().numpy()
    assert np.all((lb == lb64) | (bd < 1e-6))
    ok = lb == lb64
    d = out["dir"].cpu().numpy()
    assert np.abs(d[ok] - d64[ok]).max() < 1e-4
    p64 = oracle.mixture_pdf(raw, K, d, cosn, fp64=True)
    assert np.max(np.abs(out["pdf"].cpu().numpy() - p64) / p64) < 1e-4
    if f.cfg.selection:
        sel = out["selection"].cpu().numpy()
        assert np.abs(sel - 1 / (1 + np.exp(-raw64[:, 4 * K]))).max() < 1e-5
    # pdf of given directions
    wi = synth.uniform_sphere(np.random.default_rng(7), (8192,)).astype(np.float32)
    p = f.pdf(pos, wo, n, r, dev(wi)[0]).cpu().numpy()
    p64 = oracle.mixture_pdf(raw, K, wi, cosn, fp64=True)
    assert np.max(np.abs(p - p64) / p64) < 1e-4


def test_query_device_count(field, synth):
    """Only the first *d_count queries are written; the rest stay untouched."""
    import torch
    f, _ = field
    q = synth.wavefront(1000, seed=8)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    cnt = torch.tensor([613], dtype=torch.int32, device="cuda")
    out = {"dir": torch.full((1000, 3), 7.0, device="cuda"), "pdf": torch.full((1000,), -1.0, device="cuda"),
           "lobe": torch.full((1000,), -5, dtype=torch.int32, device="cuda")}
    f.query(pos, wo, n, r, u4, count=cnt, outputs=out)
    full = f.query(pos, wo, n, r, u4)
    assert torch.equal(out["dir"][:613], full["dir"][:613]) and torch.equal(out["pdf"][:613], full["pdf"][:613])
    assert bool((out["pdf"][613:] == -1).all()) and bool((out["lobe"][613:] == -5).all())


def block_close(g, g64, net, tol=1e-3):
    """Per block (each weight matrix, the grid table): max error <= tol * max|g64|."""
    offs = [0]
    w_in = net.n_enc_padded
    for _ in range(net.n_hidden):
        offs.append(offs[-1] + net.width * w_in)
        w_in = net.width
    offs.append(offs[-1] + net.n_out_padded * net.width)
    offs.append(net.n_params)
    for a, b in zip(offs[:-1], offs[1:]):
        ref = g64[a:b]
        scale = max(np.abs(ref).max(), 1e-30)
        err = np.abs(g[a:b] - ref).max()
        assert err <= tol * scale, (a, b, err, scale)


def test_vjp_matches_oracle(field, oracle, synth):
    f, net = field
    q = synth.wavefront(2048, seed=9)
    x = synth.featurize(q, f.cfg.input_mode)
    draw = np.random.default_rng(1).standard_normal((2048, net.n_out_padded)).astype(np.float32)
    xd, dd = dev(x, draw)
    _, dp = f.vjp(xd, dd)
    dp64 = oracle.network_backward(net, f.get_params(0).cpu().numpy(), x, draw.astype(np.float64))
    block_close(dp.cpu().numpy(), dp64, net)


@pytest.mark.parametrize("n", [4096, 40000], ids=["small", "multi-block"])
def test_train_step_gradient_and_adam(field, oracle, synth, n):
    f, net = field
    K, sel = f.cfg.n_lobes, bool(f.cfg.selection)
    f.reserve(0, n)
    fieldgt = synth.TrainField(seed=1)
    x, rec = synth.train_batch(fieldgt, n, seed=2, input_mode=f.cfg.input_mode, selection=sel)
    w0 = f.get_params(0).cpu().numpy()
    stats = f.train_step(*dev(x, rec)).cpu().numpy()
    g = f.get_gradients().cpu().numpy()
    # oracle: forward, KL adjoint (scaled by loss_scale / n), backward
    raw64 = oracle.network_forward(net, w0, x)
    graw, loss, tot = oracle.mixture_loss_grad(raw64.astype(np.float32), K, rec, 128.0, selection=sel, fp64=True)
    g64 = oracle.network_backward(net, w0, x, graw)
    block_close(g, g64, net, tol=2e-3)
    assert abs(stats[0] - tot / n) <= 1e-4 * abs(tot / n)
    assert abs(stats[1] - np.linalg.norm(g.astype(np.float64) / 128.0)) <= 1e-6 * stats[1]
    # Adam + EMA applied by the oracle to the GPU's own gradient
    w, m, v = w0.copy(), np.zeros_like(w0), np.zeros_like(w0)
    ps, ema = np.zeros(w0.size, np.uint32), w0.copy()
    oracle.adam_ema(g, 128.0, 1e-2, 0.9, 0.99, 1e-15, 1e-6, 0.95, 1, w, m, v, ps, ema, net.n_mlp_params)
    w1 = f.get_params(0).cpu().numpy()
    e1 = f.get_params(1).cpu().numpy()
    assert np.abs(w1 - w).max() <= 1e-5 * max(1.0, np.abs(w).max())
    assert np.abs(e1 - ema).max() <= 1e-5 * max(1.0, np.abs(ema).max())
    assert f.step == 1
    # grid entries with zero gradient keep their step counter and value
    untouched = (g[net.n_mlp_params:] == 0)
    assert np.array_equal(w1[net.n_mlp_params:][untouched], w0[net.n_mlp_params:][untouched])


def test_checkpoint_roundtrip(field, synth):
    import torch
    f, _ = field
    fieldgt = synth.TrainField(seed=4)
    x, rec = synth.train_batch(fieldgt, 2048, seed=5, input_mode=f.cfg.input_mode, selection=bool(f.cfg.selection))
    xd, rd = dev(x, rec)
    f.train_step(xd, rd)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ckpt.bin")
        f.save(path)
        f.train_step(xd, rd)
        w_after = f.get_params(0).clone()
        f.load(path)
        assert f.step == 1
        f.train_step(xd, rd)
        # FP32 atomics in the backward pass may reorder sums: compare to rounding
        assert torch.allclose(f.get_params(0), w_after, rtol=1e-5, atol=1e-7)


def test_capacity_and_argument_errors(nmg, synth):
    import torch
    f = nmg.GuidingField(nmg.config(nmg.PRESET_REFERENCE), max_queries=16, max_batch=16)
    q = synth.wavefront(32, seed=1)
    pos, wo, n, r, u4 = dev(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"])
    with pytest.raises(nmg.NMGError) as e:
        f.query(pos, wo, n, r, u4)
    assert e.value.status == 7  # NMG_ERR_CAPACITY
    with pytest.raises(nmg.NMGError):
        nmg.GuidingField(nmg.config(nmg.PRESET_REFERENCE, n_lobes=5))
    f.close()
    torch.cuda.synchronize()


def _read_msgpack_map(buf):
    """Just enough MessagePack to read a tcnn snapshot: a map of str keys to uint / str / bin values."""
    pos = 0

    def take(n):
        nonlocal pos
        out = buf[pos:pos + n]
        pos += n
        return out

    def value():
        t = take(1)[0]
        if t < 0x80:
            return t
        if 0xa0 <= t <= 0xbf:
            return take(t & 0x1f).decode()
        if t in (0xcc, 0xcd, 0xce, 0xcf):
            return int.from_bytes(take({0xcc: 1, 0xcd: 2, 0xce: 4, 0xcf: 8}[t]), "big")
        if t in (0xc4, 0xc5, 0xc6):
            return bytes(take(int.from_bytes(take({0xc4: 1, 0xc5: 2, 0xc6: 4}[t]), "big")))
        if t == 0xd9:
            return take(take(1)[0]).decode()
        raise ValueError(hex(t))

    t = take(1)[0]
    assert 0x80 <= t <= 0x8f
    out = {}
    for _ in range(t & 0x0f):
        k = value()
        out[k] = value()
    assert pos == len(buf)
    return out


def test_tcnn_snapshot_roundtrip(field, nmg, tmp_path):
    """tiny-cuda-nn Trainer snapshot (MessagePack of {n_params, params_binary, params_type}): the file
    holds the inference parameters in the reference's [MLP | grid] order; float snapshots restore them
    exactly, __half snapshots to their binary16 rounding; sizes and types are checked."""
    import torch
    f, _ = field
    p = f.get_params(0)
    g = torch.Generator(device="cuda").manual_seed(31)
    f.set_params(p + 0.05 * torch.randn(p.numel(), device="cuda", generator=g))
    want = f.get_params(1).cpu().numpy()
    for kind in ("float", "__half"):
        path = tmp_path / ("snap_%s.msgpack" % kind)
        f.export_tcnn(path, kind)
        obj = _read_msgpack_map(path.read_bytes())
        assert set(obj) == {"n_params", "params_binary", "params_type"}
        assert obj["n_params"] == f.n_params and obj["params_type"] == kind
        blob = np.frombuffer(obj["params_binary"], dtype=np.float32 if kind == "float" else np.float16)
        expect = want if kind == "float" else want.astype(np.float16)
        assert blob.shape == (f.n_params,) and np.array_equal(blob, expect)
        g2 = nmg.GuidingField(f.cfg)
        g2.import_tcnn(path)
        for which in (0, 1):
            assert np.array_equal(g2.get_params(which).cpu().numpy(), expect.astype(np.float32))
        g2.close()
    # a snapshot of another network is refused
    other = nmg.GuidingField(nmg.config(1 - int(f.cfg.input_mode), path=nmg.PATH_FP32))
    other.export_tcnn(tmp_path / "other.msgpack")
    with pytest.raises(nmg.NMGError):
        f.import_tcnn(tmp_path / "other.msgpack")
    other.close()
