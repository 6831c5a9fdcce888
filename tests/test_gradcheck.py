"""Gradient checks of the hand-derived adjoints (the differentiation workload:
4,096 training records, FP64 central finite differences with h = 1e-6 on 256
randomly chosen parameters, and torch autograd of the same loss).

CPU (oracle): the FP64 mixture adjoint against torch autograd of the KL loss
written in torch; the FP64 network adjoint against central differences.
GPU: the FP32 kernels through torch.autograd.Function (GuidingNetworkFn,
MixtureKLFn) against the same references.
"""
import importlib

import numpy as np
import pytest

N = 4096
H = 1e-6


def torch_loss_grad(raw, rec, K):
    import torch
    agd = importlib.import_module("neural-mixture-guiding_gb300.autograd")
    r = torch.from_numpy(np.asarray(raw, np.float64)).requires_grad_(True)
    loss = agd.kl_loss_torch(r, torch.from_numpy(np.asarray(rec, np.float64)), K)
    loss.backward()
    return float(loss.detach()), r.grad.numpy()


def test_oracle_mixture_adjoint_matches_torch_autograd(oracle, synth):
    """dL/draw of distribution.h:144-181 + train.cu:95-104 (exact kappa term) equals autograd."""
    raw, _, rec = synth.mixture_batch(512, 8, seed=31)
    # keep logits inside the exp clamp (the reference's derivative ignores the clamp, train.h:410)
    raw[:, 0:32:4] = np.clip(raw[:, 0:32:4], -9.5, 14.5)
    raw[:, 1:32:4] = np.clip(raw[:, 1:32:4], -9.5, 14.5)
    n = raw.shape[0]
    g, _, tot = oracle.mixture_loss_grad(raw, 8, rec, loss_scale=1.0, fp64=True, o=oracle.opts(kappa_poly=0))
    g = g[:, :32] * n  # loss_scale / n = 1/n: undo to get d(sum of losses)/draw
    lt, gt = torch_loss_grad(raw, rec, 8)
    assert abs(lt - tot) <= 1e-9 * abs(lt)
    err = np.abs(g - gt[:, :32]).max(axis=1)
    assert np.all(err <= 1e-8 * np.maximum(1.0, np.abs(gt).max(axis=1)))


def _fd_setup(nmg, oracle, synth, preset=1):
    cfg = nmg.config(preset, selection=0)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    rng = np.random.default_rng(5)
    params = np.zeros(net.n_params, np.float32)
    params[:net.n_mlp_params] = rng.uniform(-0.2, 0.2, net.n_mlp_params)
    params[net.n_mlp_params:] = rng.normal(0.0, 0.1, net.n_params - net.n_mlp_params)
    gt = synth.TrainField(seed=8)
    x, rec = synth.train_batch(gt, N, seed=9, input_mode=cfg.input_mode, selection=False)
    return cfg, net, params, x, rec


def _loss64(oracle, net, params, x, rec, K):
    raw = oracle.network_forward(net, params, x)
    lt, graw = torch_loss_grad(raw, rec, K)
    return lt, graw


def _pick_params(net, dparams, rng, count=256):
    mlp = rng.choice(net.n_mlp_params, count // 2, replace=False)
    touched = np.flatnonzero(dparams[net.n_mlp_params:] != 0) + net.n_mlp_params
    grid = rng.choice(touched, count - count // 2, replace=False)
    return np.concatenate([mlp, grid])


def _central_fd(oracle, net, params, x, rec, K, idx):
    out = np.zeros(len(idx))
    for j, i in enumerate(idx):
        p_plus, p_minus = params.copy(), params.copy()
        p_plus[i] = np.float32(params[i] + H)
        p_minus[i] = np.float32(params[i] - H)
        lp, _ = _loss64(oracle, net, p_plus, x, rec, K)
        lm, _ = _loss64(oracle, net, p_minus, x, rec, K)
        out[j] = (lp - lm) / (float(p_plus[i]) - float(p_minus[i]))  # the float32 step actually taken
    return out


def test_oracle_network_adjoint_vs_central_differences(nmg, oracle, synth):
    """FP64: network adjoint (MLP + hash grid) against central differences on 256 parameters."""
    cfg, net, params, x, rec = _fd_setup(nmg, oracle, synth)
    _, graw = _loss64(oracle, net, params, x, rec, cfg.n_lobes)
    dparams = oracle.network_backward(net, params, x, graw)
    idx = _pick_params(net, dparams, np.random.default_rng(11))
    fd = _central_fd(oracle, net, params, x, rec, cfg.n_lobes, idx)
    scale = np.abs(dparams[idx]).max()
    assert np.abs(fd - dparams[idx]).max() <= 1e-4 * scale, np.abs(fd - dparams[idx]).max() / scale


@pytest.mark.gpu
def test_autograd_functions_match_fd_and_fp64(nmg, oracle, synth):
    """FP32 kernels through torch.autograd.Function: the network VJP with the torch-autograd loss
    gradient, and the hand-derived mixture adjoint (MixtureKLFn) against autograd of the same loss."""
    import torch
    agd = importlib.import_module(nmg.__name__ + ".autograd")
    cfg, net, params, x, rec = _fd_setup(nmg, oracle, synth)
    field = nmg.GuidingField(nmg.config(1, selection=0, path=nmg.PATH_FP32), max_queries=N, max_batch=N)
    xd = torch.from_numpy(x).cuda()
    recd = torch.from_numpy(rec).cuda().double()
    p = torch.from_numpy(params).cuda().requires_grad_(True)
    raw = agd.GuidingNetworkFn.apply(xd, p, field)
    loss = agd.kl_loss_torch(raw.double(), recd, cfg.n_lobes)
    loss.backward()
    g_gpu = p.grad.cpu().numpy().astype(np.float64)
    # FP64 adjoint
    _, graw = _loss64(oracle, net, params, x, rec, cfg.n_lobes)
    g64 = oracle.network_backward(net, params, x, graw)
    idx = _pick_params(net, g64, np.random.default_rng(12))
    scale = np.abs(g64[idx]).max()
    assert np.abs(g_gpu[idx] - g64[idx]).max() <= 1e-3 * scale
    # the hand-derived mixture adjoint against autograd of kl_loss_torch, both on the GPU's raw outputs
    raw2 = raw.detach().clone().requires_grad_(True)
    l_hand = agd.MixtureKLFn.apply(raw2, recd.float(), cfg.n_lobes, False)
    l_hand.backward()
    raw3 = raw.detach().double().requires_grad_(True)
    agd.kl_loss_torch(raw3, recd, cfg.n_lobes).backward()
    gh, ga = raw2.grad.cpu().numpy()[:, :32], raw3.grad.cpu().numpy()[:, :32]
    assert np.all(np.abs(gh - ga).max(axis=1) <= 1e-3 * np.maximum(1.0, np.abs(ga).max(axis=1)))
    assert abs(float(l_hand.detach()) - float(loss.detach())) <= 1e-5 * abs(float(loss.detach()))
    # central differences (FP64 oracle) at 64 of the parameters
    fd = _central_fd(oracle, net, params, x, rec, cfg.n_lobes, idx[::4])
    assert np.abs(g_gpu[idx[::4]] - fd).max() <= 2e-3 * np.abs(fd).max()
    field.close()
