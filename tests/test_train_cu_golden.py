"""The oracle's featurisation and training-record extraction pinned against the
reference's own train.cu kernels.

tests/golden/train_cu_golden.npz (tests/golden/make_golden.py) holds the
outputs of generate_training_data (train.cu:14-67) and generate_inference_data
(train.cu:174-191), compiled from the reference's source as host functions and
run once per thread index, on seeded inputs with every case the kernels
branch on: delta vertices, throughputs below and exactly at M_EPSILON = 1e-5,
NaN positions / directions / outgoing directions / pdfs / MIS weights /
radiance, NaN and Inf BSDF values, zero pdfs, a training-pixel grid that runs
off the image; positions on and outside the scene box, non-unit outgoing
directions, normals on the axes. The inference inputs went through the
reference's soac-generated ScatterRayQueue, whose field arrays are stored
too."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tcu():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "train_cu_golden.npz")))


def per_depth(g):
    keys = ("L", "thp", "pos", "dir", "wi_pdf", "bsdf_pdf", "mis_weight", "delta", "bsdf_val", "wo", "normal",
            "roughness")
    return {k: list(g["rec_" + k]) for k in keys}


def test_record_extraction_matches_reference_kernel(oracle, tcu):
    """FP32 restatement vs the reference kernel: the same records in the same order; the kept set, the
    GuidedOutput rows (NaN radiance included) and the normalised positions bit for bit; the inputs that go
    through sin/cos/exp (numpy's float32 functions against the host libm) within 2 ulp of 1.0, their
    scale (each lies in [0, 1])."""
    g = tcu
    x, out = oracle.extract_records(per_depth(g), g["cur_depth"], g["offset"], g["stride"], g["train_res"],
                                    g["res"], g["aabb"], input_mode=0)
    assert x.shape == g["rec_x"].shape and len(x) > 300
    assert np.array_equal(out, g["rec_out"], equal_nan=True)
    assert np.array_equal(x[:, :3], g["rec_x"][:, :3])
    assert np.array_equal(x[:, 6:8], g["rec_x"][:, 6:8])  # normal angles times 1/pi, 1/(2 pi)
    assert np.abs(x[:, 3:] - g["rec_x"][:, 3:]).max() <= 2 * np.spacing(np.float32(1))


def test_record_filter_cases_present(tcu):
    """The fixture exercises the rules that differ between testing the radiance before and after the BSDF
    factor: records the reference keeps with a NaN (or Inf) stored radiance because only bsdfVal is bad."""
    out = tcu["rec_out"]
    assert np.isnan(out[:, 2:5]).any(axis=1).sum() >= 3
    assert np.isinf(out[:, 2:5]).any(axis=1).sum() >= 3
    assert not np.isnan(out[:, [0, 1, 5]]).any() and np.all(out[:, 5] != 0)
    assert not np.isnan(tcu["rec_x"]).any()


def test_record_filter_rule_on_planted_cases(oracle, tcu):
    """Planted in the oracle's inputs: a NaN outgoing direction drops a vertex, a NaN bsdfVal keeps it,
    a throughput exactly at 1e-5 zeroes its channel."""
    g = tcu
    rec = per_depth(g)
    cur = g["cur_depth"].copy()
    res, off, st = g["res"], g["offset"], g["stride"]
    pid = int(off[0] + off[1] * res[0])  # training pixel (0, 0)
    cur[pid] = 1
    for k in rec:
        rec[k] = [a.copy() for a in rec[k]]
    r0 = {k: rec[k][0] for k in rec}
    r0["delta"][pid] = 0
    r0["pos"][pid] = (0.1, 0.2, 0.3)
    r0["dir"][pid] = (1.0, 2.0)
    r0["wi_pdf"][pid] = 0.5
    r0["mis_weight"][pid] = 0.5
    r0["thp"][pid] = (1.0, np.float32(1e-5), 0.5)
    r0["L"][pid] = (2.0, 3.0, 4.0)
    r0["bsdf_val"][pid] = (np.nan, 1.0, 1.0)
    r0["wo"][pid] = (0.5, 0.5)
    args = (cur, off, st, g["train_res"], res, g["aabb"])
    x, out = oracle.extract_records(rec, *args)
    first = out[0]
    assert np.isnan(first[2]) and first[3] == 0.0 and first[4] == np.float32(4.0) / np.float32(0.5) * np.float32(0.5)
    r0["wo"][pid] = (np.nan, 0.5)
    x2, out2 = oracle.extract_records(rec, *args)
    assert len(out2) == len(out) - 1 and np.array_equal(out2, out[1:], equal_nan=True)
    if oracle.ref_lib() is not None:  # the reference kernel itself agrees (only where its checkout exists)
        _, rout = oracle.ref_extract_records(rec, *args)
        assert np.array_equal(rout, out2, equal_nan=True)


def test_inference_featurisation_matches_reference_kernel(oracle, nmg, tcu):
    g = tcu
    cfg = nmg.config(nmg.PRESET_REFERENCE, aabb=[float(v) for v in g["aabb"]])
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    x = oracle.featurize(net, g["soa_pos"], g["soa_wo"], g["soa_normal"], g["soa_rough"], g["aabb"])
    assert np.array_equal(x[:, :3], g["q_x"][:, :3])
    assert np.all(np.abs(x - g["q_x"]) <= 2 * np.spacing(np.abs(g["q_x"])))


def test_scatter_ray_queue_fields_are_flat_arrays(tcu):
    """The soac-generated SOA<ScatterRayWorkItem> stores sd.pos, sd.wo, sd.frame.N as packed float
    triples and sd.roughness as floats, one per queue slot: exactly the nmg_shading arrays."""
    for k, q in (("pos", "pos"), ("wo", "wo"), ("normal", "normal"), ("rough", "rough")):
        assert np.array_equal(tcu["soa_" + k], tcu["q_" + q])
