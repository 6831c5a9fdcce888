"""Host-buffer entry points (nmg_query_host, nmg_train_step_host): the
chunked, copy-overlapped pipeline returns what the device-buffer calls return
on the same inputs, for both the fused BF16 path and the plain FP32 path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", [1, 0])
def test_query_host_matches_device_query(nmg, synth, path):
    import torch
    n = 1_100_001  # four chunks, the last ragged
    f = nmg.GuidingField(nmg.config(1, path=path), max_queries=n)
    q = synth.wavefront(n, seed=404)
    keys = ("pos", "wo", "normal", "rough", "u4")
    host = {k: torch.from_numpy(np.ascontiguousarray(q[k])).pin_memory() for k in keys}
    dev = {k: v.cuda() for k, v in host.items()}
    ref = f.query(*(dev[k] for k in keys))
    out = {"dir": torch.empty((n, 3)).pin_memory(), "pdf": torch.empty(n).pin_memory(),
           "lobe": torch.empty(n, dtype=torch.int32).pin_memory(), "selection": torch.empty(n).pin_memory()}
    f.query_host(*(host[k] for k in keys), out)
    torch.cuda.synchronize()
    assert torch.equal(out["dir"], ref["dir"].cpu())
    assert torch.equal(out["pdf"], ref["pdf"].cpu())
    assert torch.equal(out["lobe"], ref["lobe"].cpu())
    assert torch.equal(out["selection"], ref["selection"].cpu())
    # pageable host memory works too (synchronous copies), and n = 0 is a no-op
    out2 = {k: torch.empty_like(v) for k, v in out.items()}
    f.query_host(*(torch.from_numpy(np.ascontiguousarray(q[k])) for k in keys), out2)
    torch.cuda.synchronize()
    assert torch.equal(out2["pdf"], out["pdf"])
    f.check_errors()
    f.close()


@pytest.mark.parametrize("path", [1, 0])
def test_train_step_host_matches_device_step(nmg, synth, path):
    import torch
    n = 50_000
    gt = synth.TrainField(seed=5)
    x, rec = synth.train_batch(gt, n, seed=6, input_mode=1, selection=True)
    a = nmg.GuidingField(nmg.config(1, path=path), max_batch=n)
    b = nmg.GuidingField(nmg.config(1, path=path), max_batch=n)
    sa = a.train_step(torch.from_numpy(x).cuda(), torch.from_numpy(rec).cuda())
    hs = torch.zeros(2, dtype=torch.float64).pin_memory()
    b.train_step_host(torch.from_numpy(x).pin_memory(), torch.from_numpy(rec).pin_memory(), stats=hs)
    torch.cuda.synchronize()
    s_dev = sa.cpu().numpy()
    assert abs(hs[0].item() - s_dev[0]) <= 1e-12 * abs(s_dev[0])
    assert abs(hs[1].item() - s_dev[1]) <= 1e-6 * abs(s_dev[1])  # gradient norm: atomics in the grid scatter
    # Adam's first step moves every touched parameter by lr * sign(g): identical except where the grid
    # gradient's atomics, summed in another order, land on the other side of zero
    pa, pb = a.get_params(0), b.get_params(0)
    assert float(((pa - pb).abs() > 1e-6).float().mean()) <= 1e-5
    assert a.step == b.step == 1
    for g in (a, b):
        g.check_errors()
        g.close()


def test_host_steps_interleaved_match_device_steps(nmg, synth):
    """Alternating host-buffer training steps and queries, each on new inputs (so a copy that overtook
    the previous kernel's use of the staging would feed stale data): the results follow the device-buffer
    calls on the same inputs, up to the float-atomic order of the training steps."""
    import torch
    n, nb = 600_000, 40_000
    keys = ("pos", "wo", "normal", "rough", "u4")
    a = nmg.GuidingField(nmg.config(1, path=1), max_queries=n, max_batch=nb)
    b = nmg.GuidingField(nmg.config(1, path=1), max_queries=n, max_batch=nb)
    gt = synth.TrainField(seed=50)
    outs = []
    for it in range(3):
        q = synth.wavefront(n, seed=51 + it)
        x, rec = synth.train_batch(gt, nb, seed=61 + it, input_mode=1, selection=True)
        hq = {k: torch.from_numpy(np.ascontiguousarray(q[k])).pin_memory() for k in keys}
        hx, hr = torch.from_numpy(x).pin_memory(), torch.from_numpy(rec).pin_memory()
        a.train_step_host(hx, hr)
        ho = {"dir": torch.empty((n, 3)).pin_memory(), "pdf": torch.empty(n).pin_memory(),
              "lobe": torch.empty(n, dtype=torch.int32).pin_memory()}
        a.query_host(*(hq[k] for k in keys), ho)
        b.train_step(hx.cuda(), hr.cuda())
        ref = b.query(*(hq[k].cuda() for k in keys))
        outs.append((ho, ref))
    torch.cuda.synchronize()
    for ho, ref in outs:
        same = ho["lobe"] == ref["lobe"].cpu()
        assert float(same.float().mean()) >= 0.999
        rel = ((ho["pdf"] - ref["pdf"].cpu()) / ref["pdf"].cpu())[same]
        assert float(rel.pow(2).mean().sqrt()) <= 1e-3
    a.check_errors()
    for f in (a, b):
        f.close()


def test_query_host_slots_chunks_and_output_kinds(nmg, synth):
    """Queued query_host calls on different inputs (the two input staging slots alternate, the third
    call reuses the first slot while nothing has synchronised), at 1, 2, 3 and 8 chunks and automatic
    (4 chunks for the first call on the idle stream, 1 for the two queued behind it), with outputs
    in pinned memory (written by the kernel through the mapping), in pageable memory (staged and
    copied back) and mixed (one pageable output stages them all): every result equals the
    device-buffer query on the same inputs."""
    import torch
    n = 800_003
    keys = ("pos", "wo", "normal", "rough", "u4")
    f = nmg.GuidingField(nmg.config(1, path=1), max_queries=n)
    assert f.host_chunks == 4
    with pytest.raises(nmg.NMGError):
        f.set_host_chunks(9)
    with pytest.raises(nmg.NMGError):
        f.set_host_chunks(-1)
    qs = [synth.wavefront(n, seed=900 + i) for i in range(3)]
    hq = [{k: torch.from_numpy(np.ascontiguousarray(q[k])).pin_memory() for k in keys} for q in qs]
    refs = [f.query(*(h[k].cuda() for k in keys)) for h in hq]
    torch.cuda.synchronize()
    refs = [{k: v.cpu() for k, v in r.items() if v is not None} for r in refs]

    def outputs(kind):
        o = {"dir": torch.empty((n, 3)), "pdf": torch.empty(n), "lobe": torch.empty(n, dtype=torch.int32)}
        if kind == "pinned":
            o = {k: v.pin_memory() for k, v in o.items()}
        elif kind == "mixed":
            o = {k: (v if k == "pdf" else v.pin_memory()) for k, v in o.items()}
        return o

    for chunks in (1, 2, 3, 8, 0):
        f.set_host_chunks(chunks)
        assert f.host_chunks == (chunks or 4)
        for kind in ("pinned", "pageable", "mixed"):
            outs = [outputs(kind) for _ in qs]
            torch.cuda.synchronize()
            for h, o in zip(hq, outs):
                f.query_host(*(h[k] for k in keys), o)
            torch.cuda.synchronize()
            for o, r in zip(outs, refs):
                for k in ("dir", "pdf", "lobe"):
                    assert torch.equal(o[k], r[k]), (chunks, kind, k)
    f.check_errors()
    f.close()
