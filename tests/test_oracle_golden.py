"""The oracle pinned against the reference's own mixture code.

tests/golden/mixture_golden.npz holds outputs of the reference's
distribution.h / vmf.h / train.h compiled on the host (make_golden.py). The
FP32 restatement must reproduce them bit for bit; the FP64 oracle must agree
within the conditioning of FP32 arithmetic."""
import numpy as np
import pytest


def test_fp32_sample_bit_exact(oracle, golden):
    K = int(golden["K"])
    d, p, lb = oracle.mixture_sample(golden["raw"], K, golden["u4"], fp64=False)
    assert np.array_equal(lb, golden["lobe"])
    assert np.array_equal(d.astype(np.float32), golden["dir"])
    assert np.array_equal(p.astype(np.float32), golden["pdf"])


def test_fp32_sample_cosine_bit_exact(oracle, golden):
    K = int(golden["K"])
    d, p, lb = oracle.mixture_sample(golden["raw"], K, golden["u4"], golden["cosn"], fp64=False)
    assert np.array_equal(lb, golden["lobe_cos"])
    assert np.array_equal(d.astype(np.float32), golden["dir_cos"])
    assert np.array_equal(p.astype(np.float32), golden["pdf_cos"])


def test_fp32_pdf_bit_exact(oracle, golden):
    K = int(golden["K"])
    p = oracle.mixture_pdf(golden["raw"], K, golden["wi"], fp64=False)
    pc = oracle.mixture_pdf(golden["raw"], K, golden["wi"], golden["cosn"], fp64=False)
    assert np.array_equal(p.astype(np.float32), golden["pdf_eval"])
    assert np.array_equal(pc.astype(np.float32), golden["pdf_eval_cos"])


def test_fp32_loss_grad_bit_exact_with_half_storage(oracle, golden):
    K = int(golden["K"])
    raw_h = golden["raw"].astype(np.float16).astype(np.float32)  # __half network outputs
    g, loss, _ = oracle.mixture_loss_grad(raw_h, K, golden["rec"], float(golden["loss_scale"]), fp64=False,
                                          o=oracle.opts(half_grad=1))
    assert np.array_equal(loss.astype(np.float32), golden["loss"])
    assert np.array_equal(g[:, :4 * K].astype(np.float32), golden["grad"][:, :4 * K])


def test_fp64_close_to_reference(oracle, golden):
    K = int(golden["K"])
    raw = golden["raw"]
    d, p, lb = oracle.mixture_sample(raw, K, golden["u4"], fp64=True)
    bd = oracle.boundary_distance(raw, K, golden["u4"])
    ok = bd > 1e-6
    assert np.array_equal(lb[ok], golden["lobe"][ok])
    assert np.abs(d[ok] - golden["dir"][ok]).max() < 1e-4
    pe = oracle.mixture_pdf(raw, K, golden["wi"], fp64=True)
    rel = np.abs(pe - golden["pdf_eval"]) / pe
    assert np.median(rel) < 1e-6 and rel.max() < 2e-3


def test_exact_kappa_switch_differs_only_below_one(oracle, synth):
    raw, _, rec = synth.mixture_batch(2048, 8, seed=11)
    g_poly, _, _ = oracle.mixture_loss_grad(raw, 8, rec, fp64=True, o=oracle.opts(kappa_poly=1))
    g_exact, _, _ = oracle.mixture_loss_grad(raw, 8, rec, fp64=True, o=oracle.opts(kappa_poly=0))
    kappa = np.exp(np.clip(raw[:, 1:32:4], -10, 15))
    diff = np.abs(g_poly[:, 1:32:4] - g_exact[:, 1:32:4])
    assert diff[kappa >= 1.0].max() == 0.0
    assert diff[kappa < 1.0].max() > 0.0


def test_selection_variant_reduces_to_mixture_when_sel_is_one(oracle, synth):
    raw, _, rec = synth.mixture_batch(512, 8, seed=3, selection=True)
    raw[:, 32] = 40.0  # logistic -> 1: pdf = mixture pdf
    g, loss, _ = oracle.mixture_loss_grad(raw, 8, rec, selection=True, fp64=True)
    assert np.all(np.isfinite(g)) and np.all(np.isfinite(loss))
    assert np.abs(g[:, 32]).max() < 1e-12
