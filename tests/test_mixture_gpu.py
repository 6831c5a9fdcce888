"""Parity of the CUDA mixture kernels (nmg_mixture_*) with the oracle.

Tolerances (FP32 path against the FP64 oracle):
  * lobe index: identical, except for queries whose u_lobe lies within 1e-6
    of an FP64 CDF boundary (the FP32 weights move a boundary by ~1e-7);
    those are counted and must be rare.
  * direction: |d_gpu - d_fp64|_inf <= 1e-4.
  * pdf: evaluated by both at the GPU's direction, relative error
    <= 1e-4 + 4e-7 * kappa_max. An FP32 direction is only known to ~6e-8,
    which the lobe exponent kappa*(cos-1) amplifies by kappa; below
    kappa ~ 250 the bound is 1e-4.
  * KL gradient: per row, max|g_gpu - g_fp64| <= 1e-3 * max(1, max|g_fp64|);
    loss relative 1e-5; FP64 loss sum relative 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 65536  # the mixture workload's query count


def to_dev(*arrs):
    import torch
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def kappa_max(raw, K, cosine):
    k = np.exp(np.clip(raw[:, 1:4 * K:4].astype(np.float64), -10, 15)).max(axis=1)
    return k + 2.2 if cosine else k


def check_sample(nmg, oracle, raw, u4, K, cosn=None, limit_near=True):
    r, u, c = to_dev(raw, u4, cosn)
    d, p, lb = nmg.mixture_sample(r, u, K, cos_normal=c)
    d, p, lb = d.cpu().numpy(), p.cpu().numpy(), lb.cpu().numpy()
    d64, _, lb64 = oracle.mixture_sample(raw, K, u4, cosn, fp64=True)
    bd = oracle.boundary_distance(raw, K, u4, cosn)
    near = bd < 1e-6
    mism = lb != lb64
    assert not np.any(mism & ~near), "lobe mismatch away from a CDF boundary"
    if limit_near:  # random uniforms rarely land within 1e-6 of a boundary
        assert near.sum() <= max(4, len(raw) // 5000)
    ok = ~mism
    assert np.abs(d[ok] - d64[ok]).max() <= 1e-4
    assert np.abs(np.linalg.norm(d, axis=1) - 1).max() < 1e-5
    p64 = oracle.mixture_pdf(raw, K, d, cosn, fp64=True)
    rel = np.abs(p - p64) / p64
    tol = 1e-4 + 4e-7 * kappa_max(raw, K, cosn is not None)
    assert np.all(rel <= tol), (rel.max(), np.argmax(rel / tol))
    return d, p, lb


@pytest.mark.parametrize("K", [8, 16])
def test_sample_and_pdf_vs_fp64(nmg, oracle, synth, K):
    raw, u4, _ = synth.mixture_batch(N, K, seed=7272)
    check_sample(nmg, oracle, raw, u4, K)


def test_sample_cosine_lobe_vs_fp64(nmg, oracle, synth):
    raw, u4, _ = synth.mixture_batch(N, 8, seed=1)
    n = synth.uniform_sphere(np.random.default_rng(2), (N,)).astype(np.float32)
    check_sample(nmg, oracle, raw, u4, 8, n)


def test_golden_reference_vectors(nmg, oracle, golden):
    """Against the reference's own FP32 outputs (lobe index bit-exact except at boundaries)."""
    K = int(golden["K"])
    for cos in (False, True):
        cosn = golden["cosn"] if cos else None
        d, p, lb = check_sample(nmg, oracle, golden["raw"], golden["u4"], K, cosn, limit_near=False)
        ref_lb = golden["lobe_cos" if cos else "lobe"]
        bd = oracle.boundary_distance(golden["raw"], K, golden["u4"], cosn)
        assert np.all((lb == ref_lb) | (bd < 1e-6))


def test_pdf_at_given_directions(nmg, oracle, synth, golden):
    raw, _, _ = synth.mixture_batch(N, 8, seed=5)
    wi = synth.uniform_sphere(np.random.default_rng(6), (N,)).astype(np.float32)
    r, w = to_dev(raw, wi)
    p = nmg.mixture_pdf(r, w, 8).cpu().numpy()
    p64 = oracle.mixture_pdf(raw, 8, wi, fp64=True)
    rel = np.abs(p - p64) / p64
    assert np.all(rel <= 1e-4 + 4e-7 * kappa_max(raw, 8, False))
    # reference golden pdf evaluations
    r, w, c = to_dev(golden["raw"], golden["wi"], golden["cosn"])
    pg = nmg.mixture_pdf(r, w, 8, cos_normal=c).cpu().numpy()
    relg = np.abs(pg - golden["pdf_eval_cos"]) / golden["pdf_eval_cos"]
    assert np.median(relg) < 1e-5 and relg.max() < 5e-3


@pytest.mark.parametrize("K,selection,kappa_poly", [(8, False, True), (8, False, False), (16, False, True),
                                                    (7, True, True), (8, True, True)])
def test_loss_grad_vs_fp64(nmg, oracle, synth, K, selection, kappa_poly):
    raw, _, rec = synth.mixture_batch(N, K, seed=9, selection=selection)
    r, rc = to_dev(raw, rec)
    g, loss, tot = nmg.mixture_loss_grad(r, rc, K, 128.0, selection=selection, kappa_poly=kappa_poly)
    g, loss, tot = g.cpu().numpy(), loss.cpu().numpy(), float(tot.cpu().numpy()[0])
    g64, l64, t64 = oracle.mixture_loss_grad(raw, K, rec, 128.0, selection=selection, fp64=True,
                                             o=oracle.opts(kappa_poly=int(kappa_poly)))
    nout = 4 * K + (1 if selection else 0)
    err = np.abs(g[:, :nout] - g64[:, :nout]).max(axis=1)
    scale = np.maximum(1.0, np.abs(g64[:, :nout]).max(axis=1))
    assert np.all(err <= 1e-3 * scale), err.max()
    assert np.all(g[:, nout:] == 0)
    # loss = -(L/p) log q: its error is (L/p) dq/q (and, with learned selection where p is the model's
    # own pdf, (L/p)(1 + |log p|) dp/p), so the bound scales with L/p, not with the loss itself
    Li = (rec[:, 2] + rec[:, 3] + rec[:, 4]) / 3.0
    if selection:
        wi = np.stack([np.sin(rec[:, 0]) * np.cos(rec[:, 1]), np.sin(rec[:, 0]) * np.sin(rec[:, 1]),
                       np.cos(rec[:, 0])], axis=1)
        q64 = oracle.mixture_pdf(raw, K, wi, fp64=True)
        sel = 1.0 / (1.0 + np.exp(-raw[:, 4 * K].astype(np.float64)))
        p = sel * (q64 + 1e-5) + (1 - sel) * rec[:, 6]
        wscale = Li / p * (1.0 + np.abs(np.log(p)))
    else:
        wscale = Li / (rec[:, 5] + 1e-5)
    kmax = kappa_max(raw, K, False)
    assert np.all(np.abs(loss - l64) <= wscale * (1e-5 + 4e-7 * kmax) + 1e-6 * np.abs(l64))
    assert abs(tot - t64) <= 1e-5 * abs(t64) + 1e-6


def test_loss_grad_golden_half_reference(nmg, oracle, golden):
    """GPU FP32 gradient against the reference's __half-stored gradient.

    The reference rounds the mixture gradient to __half before and after the
    chain-rule products (train.cu:91-103); that rounding is the measured
    difference between the golden values and the FP64 oracle, and the GPU's
    FP32 result must lie within it (plus FP32 conditioning)."""
    K = int(golden["K"])
    raw_h = golden["raw"].astype(np.float16).astype(np.float32)
    r, rc = to_dev(raw_h, golden["rec"])
    g, loss, _ = nmg.mixture_loss_grad(r, rc, K, float(golden["loss_scale"]))
    g = g.cpu().numpy()[:, :4 * K]
    ref = golden["grad"][:, :4 * K]
    g64, l64, _ = oracle.mixture_loss_grad(raw_h, K, golden["rec"], float(golden["loss_scale"]), fp64=True)
    g64 = g64[:, :4 * K]
    kmax = kappa_max(raw_h, K, False)[:, None]
    # FP32 error of dF/dlambda = (vmf_s - q)/total scales with the row's largest terms (cancellation)
    tol = np.abs(ref - g64) * 1.01 + (2e-5 + 8e-7 * kmax) * np.abs(g64).max(axis=1, keepdims=True)
    assert np.all(np.abs(g - ref) <= tol)
    rec = golden["rec"]
    wscale = ((rec[:, 2] + rec[:, 3] + rec[:, 4]) / 3.0) / (rec[:, 5] + 1e-5)
    errL = np.abs(loss.cpu().numpy() - golden["loss"])
    assert np.all(errL <= np.abs(golden["loss"] - l64) * 1.01 + wscale * (1e-5 + 8e-7 * kmax[:, 0]) + 1e-6)


def test_empty_and_ragged_batches(nmg, oracle, synth):
    import torch
    raw, u4, rec = synth.mixture_batch(1000, 8, seed=4)
    for n in (1, 7, 129, 1000):
        check_sample(nmg, oracle, raw[:n], u4[:n], 8)
    e = torch.empty((0, 32), device="cuda")
    d, p, _ = nmg.mixture_sample(e, torch.empty((0, 4), device="cuda"), 8)
    assert d.shape == (0, 3) and p.shape == (0,)
    g, l, tot = nmg.mixture_loss_grad(e, torch.empty((0, 6), device="cuda"), 8)
    assert float(tot.cpu()[0]) == 0.0


def test_softplus_kappa(nmg, oracle, synth):
    raw, u4, rec = synth.mixture_batch(8192, 8, seed=12)
    raw[:, 1:32:4] = np.random.default_rng(1).uniform(-14, 6, (8192, 8))  # reaches kappa < 1e-5 (uniform lobes)
    r, u, rc = to_dev(raw, u4, rec)
    d, p, lb = nmg.mixture_sample(r, u, 8, kappa_softplus=True)
    d64, _, lb64 = oracle.mixture_sample(raw, 8, u4, fp64=True, o=oracle.opts(kappa_softplus=1))
    # a lobe whose kappa is within 1% of the 1e-5 switch to uniform sampling (vmf.h:49) may take either branch
    kap = np.logaddexp(0.0, raw[:, 1:32:4].astype(np.float64))
    lbg = lb.cpu().numpy()
    near_switch = np.abs(kap[np.arange(len(lbg)), lbg] / 1e-5 - 1) < 1e-2
    ok = (lbg == lb64) & ~near_switch
    assert ok.mean() > 0.998
    assert np.abs(d.cpu().numpy()[ok] - d64[ok]).max() <= 1e-4
    # the pdf at the sampled direction, uniform lobes (kappa < 1e-5: 1/4pi) included; kappa <= 6.0025
    dg = d.cpu().numpy()
    p64 = oracle.mixture_pdf(raw, 8, dg, fp64=True, o=oracle.opts(kappa_softplus=1))
    assert np.all(np.abs(p.cpu().numpy() - p64) / p64 <= 1e-4)
    pw = nmg.mixture_pdf(r, d, 8, kappa_softplus=True).cpu().numpy()
    assert np.all(np.abs(pw - p64) / p64 <= 1e-4)
    g, _, _ = nmg.mixture_loss_grad(r, rc, 8, kappa_softplus=True)
    g64, _, _ = oracle.mixture_loss_grad(raw, 8, rec, fp64=True, o=oracle.opts(kappa_softplus=1))
    err = np.abs(g.cpu().numpy()[:, :32] - g64[:, :32]).max(axis=1)
    assert np.all(err <= 1e-3 * np.maximum(1.0, np.abs(g64[:, :32]).max(axis=1)))


@pytest.mark.parametrize("K", [4, 7, 8])
def test_lobe_counts_and_ragged_sizes(nmg, oracle, synth, K):
    """Every compiled lobe count through sample, pdf and loss/gradient at sizes that leave a
    partial block, a partial lane pair round and a partial last round of the resident grid: the
    kernels prefetch each thread's next query and must stop at n. Tolerances as above."""
    raw, u4, rec = synth.mixture_batch(5000, K, seed=21)
    for n in (1, 129, 5000):
        check_sample(nmg, oracle, raw[:n], u4[:n], K)
        wi = synth.uniform_sphere(np.random.default_rng(n), (n,)).astype(np.float32)
        r, rc, w = to_dev(raw[:n], rec[:n], wi)
        p = nmg.mixture_pdf(r, w, K).cpu().numpy()
        p64 = oracle.mixture_pdf(raw[:n], K, wi, fp64=True)
        # a uniform direction far from every concentrated lobe has a density below FP32's normal
        # range (e^{kappa (cos - 1)}, kappa up to 1000), which the hardware exponential flushes to 0:
        # relative error where the density is representable, absolute error below that
        live = p64 > 1e-20
        rel = np.abs(p - p64)[live] / p64[live]
        assert np.all(rel <= 1e-4 + 4e-7 * kappa_max(raw[:n], K, False)[live]), rel.max()
        assert np.all(np.abs(p - p64)[~live] <= 1e-20)
        g, loss, tot = nmg.mixture_loss_grad(r, rc, K)
        g64, l64, t64 = oracle.mixture_loss_grad(raw[:n], K, rec[:n], fp64=True)
        nout = 4 * K
        err = np.abs(g.cpu().numpy()[:, :nout] - g64[:, :nout]).max(axis=1)
        assert np.all(err <= 1e-3 * np.maximum(1.0, np.abs(g64[:, :nout]).max(axis=1))), err.max()
        assert abs(float(tot.cpu()[0]) - t64) <= 1e-5 * abs(t64) + 1e-6


def test_row_alignment_paths_agree(nmg, synth):
    """Raw rows 32-byte aligned (sampling and loss read them with 32-byte loads) and rows starting 16
    bytes into an allocation (16-byte loads): the same directions, pdfs, lobes and gradients."""
    import torch
    raw, u4, rec = synth.mixture_batch(10_001, 8, seed=77)
    r, u, rc = to_dev(raw, u4, rec)
    flat = torch.empty(r.numel() + 4, device="cuda")
    r_off = flat[4:].view_as(r)
    r_off.copy_(r)
    assert r.data_ptr() % 32 == 0 and r_off.data_ptr() % 32 == 16
    d0, p0, l0 = nmg.mixture_sample(r, u, 8)
    d1, p1, l1 = nmg.mixture_sample(r_off, u, 8)
    assert torch.equal(d0, d1) and torch.equal(p0, p1) and torch.equal(l0, l1)
    g0, s0, t0 = nmg.mixture_loss_grad(r, rc, 8)
    g1, s1, t1 = nmg.mixture_loss_grad(r_off, rc, 8)
    assert torch.equal(g0, g1) and torch.equal(s0, s1)
    # the FP64 loss sum may add the same per-query losses in another block order
    assert abs(float(t0.cpu()[0]) - float(t1.cpu()[0])) <= 1e-12 * abs(float(t0.cpu()[0]))
