"""The network half of the oracle pinned against tiny-cuda-nn 1.7's own code.

tests/golden/tcnn_golden.npz (tests/golden/make_golden.py) holds outputs of
the reference's vendored tiny-cuda-nn, compiled from its source and run on
the host (oracle/ref_tcnn_kernels.cu, oracle/ref_tcnn_layout.cu), for the
hash-grid and the reference (dense grid, smoothstep) networks:
  * GridEncodingTemplated's level offsets and parameter count;
  * kernel_grid features and kernel_grid_backward table gradients for a table
    given by a fixed integer formula (positions on box corners, level-0
    vertices and just below 1 included);
  * kernel_sh (degrees 2 and 4) and kernel_one_blob_soa (4 bins);
  * three EMA(Adam) steps with the reference's optimiser settings;
  * Trainer snapshots written by the reference's nlohmann::json (checked
    against the library's own exporter in test_tcnn_snapshot_gpu.py).

Tolerances: offsets and counts exact; encodings 3e-7 absolute (tcnn
evaluates in FP32, the oracle in FP64; features and table values lie within
+-0.5); the grid gradient 1e-6 absolute with the same support up to entries
whose FP32 corner weight rounds to zero (below 1e-7 in FP64); Adam's weights,
moments and step counters bit for bit (both FP32, same operation order); the
EMA within the FP16 rounding of the weights it filters (tcnn filters the
16-bit network weights, the oracle the FP32 master weights: a documented
deviation)."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def tg():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "tcnn_golden.npz")))


PRESETS = [("hash", 1), ("dense", 0)]


@pytest.mark.parametrize("tag,preset", PRESETS)
def test_grid_layout_matches_tcnn(nmg, oracle, tg, tag, preset):
    cfg = nmg.config(preset)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    L = int(cfg.grid_levels)
    assert np.array_equal(np.array(net.grid_offset[:L + 1], np.uint32), tg[tag + "_offsets"])
    assert net.n_grid_params == int(tg[tag + "_n_params"])
    info = nmg.config_info(cfg)
    assert info.n_grid_params == int(tg[tag + "_n_params"])
    assert info.grid_entries == int(tg[tag + "_offsets"][-1])


@pytest.mark.parametrize("tag,preset", PRESETS)
def test_grid_encoding_matches_tcnn(nmg, oracle, tg, tag, preset):
    cfg = nmg.config(preset)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    mg = _make_golden()
    F, L = int(cfg.grid_features), int(cfg.grid_levels)
    params = np.zeros(net.n_params, np.float32)
    params[net.n_mlp_params:] = mg.table_values(net.n_grid_params)
    pos = tg[tag + "_pos"]
    x = np.zeros((len(pos), net.n_input), np.float32)
    x[:, :3] = pos
    x[:, 3:] = 0.5
    _, enc = oracle.network_forward(net, params, x, want_enc=True)
    assert np.abs(enc[:, :L * F] - tg[tag + "_features"]).max() <= 3e-7


@pytest.mark.parametrize("tag,preset", PRESETS)
def test_grid_backward_matches_tcnn(nmg, oracle, tg, tag, preset):
    cfg = nmg.config(preset)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    F, L = int(cfg.grid_features), int(cfg.grid_levels)
    pos, dl = tg[tag + "_bwd_pos"], tg[tag + "_dl_dy"]
    x = np.zeros((len(pos), net.n_input), np.float32)
    x[:, :3] = pos
    denc = np.zeros((len(pos), net.n_enc_padded))
    denc[:, :L * F] = dl
    g = oracle.grid_backward(net, x, denc)
    ref = np.zeros_like(g)
    ref[tg[tag + "_grad_index"]] = tg[tag + "_grad_value"]
    assert np.abs(g - ref).max() <= 1e-6
    only_ours = (g != 0) & (ref == 0)
    assert np.abs(g[only_ours]).max(initial=0.0) <= 1e-7
    assert not ((g == 0) & (ref != 0)).any()


def test_spherical_harmonics_match_tcnn(oracle, tg):
    x = tg["sh_in"]
    net = oracle.make_net(input_mode=1, grid_hash=0, grid_levels=1, grid_feats=2, grid_log2_T=10, grid_base_res=2,
                          grid_scale=1.5, grid_smoothstep=0, sh_degree=4, oneblob_bins=4, width=64, n_hidden=3,
                          n_out=32)
    rows = np.zeros((len(x), net.n_input), np.float32)
    rows[:, 3:6] = x
    rows[:, 6:9] = x
    params = np.zeros(net.n_params, np.float32)
    _, enc = oracle.network_forward(net, params, rows, want_enc=True)
    o = net.grid_levels * net.grid_feats
    assert np.abs(enc[:, o:o + 16] - tg["sh4"]).max() <= 3e-7
    net2 = oracle.make_net(input_mode=0, grid_hash=0, grid_levels=1, grid_feats=4, grid_log2_T=10, grid_base_res=2,
                           grid_scale=1.5, grid_smoothstep=0, sh_degree=2, oneblob_bins=4, width=64, n_hidden=3,
                           n_out=32)
    rows2 = np.zeros((len(x), net2.n_input), np.float32)
    rows2[:, 3:6] = x
    _, enc2 = oracle.network_forward(net2, np.zeros(net2.n_params, np.float32), rows2, want_enc=True)
    o2 = net2.grid_levels * net2.grid_feats
    assert np.abs(enc2[:, o2:o2 + 4] - tg["sh2"]).max() <= 3e-7


def test_oneblob_matches_tcnn(oracle, tg):
    v = tg["oneblob_in"]
    net = oracle.make_net(input_mode=0, grid_hash=0, grid_levels=1, grid_feats=4, grid_log2_T=10, grid_base_res=2,
                          grid_scale=1.5, grid_smoothstep=0, sh_degree=2, oneblob_bins=4, width=64, n_hidden=3,
                          n_out=32)
    rows = np.zeros((len(v), net.n_input), np.float32)
    rows[:, 3:6] = 0.5
    rows[:, 6:9] = v
    _, enc = oracle.network_forward(net, np.zeros(net.n_params, np.float32), rows, want_enc=True)
    o = net.grid_levels * net.grid_feats + 4
    assert np.abs(enc[:, o:o + 12] - tg["oneblob4"]).max() <= 3e-7


def test_adam_ema_matches_tcnn(oracle, tg):
    """The oracle's Adam + EMA (base.json: lr 1e-2, betas 0.9 / 0.99, eps 1e-15, l2 1e-6, EMA 0.95) against
    tcnn's adam_step and its EMA, three steps."""
    n_mat = int(tg["adam_n_matrix"])
    w = tg["adam_w0"].copy()
    m, v = np.zeros_like(w), np.zeros_like(w)
    ps, ema = np.zeros(w.size, np.uint32), np.zeros_like(w)
    for k, g in enumerate(tg["adam_grads"]):
        oracle.adam_ema(g.astype(np.float32), 128.0, 1e-2, 0.9, 0.99, 1e-15, 1e-6, 0.95, k + 1, w, m, v, ps, ema, n_mat)
    assert np.array_equal(w, tg["adam_full_w_full"])
    assert np.array_equal(m, tg["adam_full_m"])
    assert np.array_equal(v, tg["adam_full_v"])
    assert np.array_equal(ps, tg["adam_full_psteps"])
    # tcnn filters the __half copy of the weights: each averaged weight differs by its FP16 rounding,
    # at most 2^-11 of its size, and a weight moves by at most ~lr per Adam step (|m| / sqrt(v) <= 1
    # after bias correction), so the weights averaged over three steps are below |w0| + 0.03
    tol = 2.0 ** -11 * (np.abs(tg["adam_w0"]) + 0.03) + 1e-7
    assert np.all(np.abs(ema - tg["adam_full_ema_tmp"]) <= tol)
    # the half-precision EMA (tcnn's default) stores the same average rounded to __half
    assert np.all(np.abs(ema - tg["adam_half_ema16"]) <= 2 * tol)
