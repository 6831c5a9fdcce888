"""The fused tensor-core path (tcgen05 MLP, BF16 or FP16 operands, FP32
accumulate) against the FP64 oracle.

  * raw network outputs: compared with the FP64 oracle evaluated on the
    same 16-bit-rounded weights and grid table, so the remaining difference
    is the rounding of encoded features and hidden activations to 16 bits
    (2^-9 relative for BF16, 2^-11 for FP16) accumulated over the layers:
    max |err| <= 4e-2 (BF16) / 1e-2 (FP16) of max |y|, RMS <= 6e-3 / 2e-3 of RMS y.
    A wrong operand layout or descriptor gives O(1) errors.
  * mixture stage (fast-math FP32 on the fused kernel's own raw outputs):
    lobe index as the FP32 path, direction 1e-3, pdf relative 1e-3
    (+ 4e-7 kappa_max conditioning).
"""
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
    w16 = round16(f.get_params(1).cpu().numpy(), fp16)
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
    # the raw outputs of the query equal those of infer_raw on the featurised inputs
    x = f.featurize(pos, wo, n, r)
    raw2 = f.infer_raw(x, which=1).cpu().numpy()
    assert np.abs(raw - raw2).max() <= 1e-6 * max(1.0, np.abs(raw2).max())
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
