"""The guided query fed from the reference's own wavefront queue layout.

The reference's integrator featurises the shading points of its
ScatterRayQueue (generate_inference_data, train.cu:174-191), a
soac-generated SOA<ScatterRayWorkItem> (workitem.soa:89-94) whose leaves
sd.pos, sd.wo, sd.frame.N and sd.roughness are flat device arrays.
tests/golden/train_cu_golden.npz (tests/golden/make_golden.py) holds those
leaves exactly as the reference's SOA stored them after its own push(), and
the rows the reference's kernel computed from them. Here the leaves go
unchanged to nmg_featurize and nmg_query (plain FP32 path).

Tolerances: positions bit for bit; the inputs computed through
sqrt/acos/atan2/exp (device functions against the host libm the reference
was run with) within 2 ulp of 1.0, their scale; raw outputs of the query as
the FP32 field tests, 1e-4 * max(1, |y|), against the FP64 network on the
reference's rows."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tcu():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "train_cu_golden.npz")))


def leaves(g):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(g[k])).cuda()
            for k in ("soa_pos", "soa_wo", "soa_normal", "soa_rough")]


def test_featurize_queue_leaves_vs_reference_kernel(nmg, tcu):
    g = tcu
    f = nmg.GuidingField(nmg.config(nmg.PRESET_REFERENCE, path=nmg.PATH_FP32, aabb=[float(v) for v in g["aabb"]]),
                         max_queries=len(g["q_x"]))
    x = f.featurize(*leaves(g)).cpu().numpy()
    assert np.array_equal(x[:, :3], g["q_x"][:, :3])
    assert np.abs(x - g["q_x"]).max() <= 2 * np.spacing(np.float32(1))
    f.check_errors()
    f.close()


def test_query_from_queue_leaves(nmg, oracle, tcu):
    import torch
    g = tcu
    cfg = nmg.config(nmg.PRESET_REFERENCE, path=nmg.PATH_FP32, aabb=[float(v) for v in g["aabb"]])
    n = len(g["q_x"])
    f = nmg.GuidingField(cfg, max_queries=n)
    net = oracle.make_net(**nmg.oracle_net_spec(cfg))
    p = f.get_params(0)
    p[int(f.info.n_mlp_params):] = 0.3 * torch.randn(p.numel() - int(f.info.n_mlp_params), device="cuda",
                                                      generator=torch.Generator(device="cuda").manual_seed(3))
    f.set_params(p)
    u4 = torch.rand((n, 4), device="cuda", generator=torch.Generator(device="cuda").manual_seed(4))
    out = f.query(*leaves(g), u4, want_raw=True)
    raw = out["raw"].cpu().numpy()
    raw64 = oracle.network_forward(net, f.get_params(1).cpu().numpy(), g["q_x"])
    nu = net.n_out_padded
    assert np.abs(raw[:, :nu] - raw64[:, :nu]).max() <= 1e-4 * max(1.0, np.abs(raw64).max())
    assert np.all(np.isfinite(out["pdf"].cpu().numpy())) and np.all(out["pdf"].cpu().numpy() > 0)
    f.check_errors()
    f.close()
