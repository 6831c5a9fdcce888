"""Training at 2^20 records per step with activations recomputed instead of
stored: the fused BF16 step's device footprint (parameters, Adam state,
weight copies, workspaces) does not depend on the batch, the step allocates
nothing, and the plain FP32 path's stored activations are what the fused
path saves."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 20


def test_train_2pow20_recomputes_activations(nmg, synth):
    import torch
    gt = synth.TrainField(seed=3)
    x, rec = synth.train_batch(gt, N, seed=4, input_mode=1, selection=True)
    xd, rd = torch.from_numpy(x).cuda(), torch.from_numpy(rec).cuda()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    f = nmg.GuidingField(nmg.config(1, path=nmg.PATH_BF16), max_queries=0, max_batch=N)
    small = nmg.GuidingField(nmg.config(1, path=nmg.PATH_BF16), max_queries=0, max_batch=1 << 12)
    stats = torch.zeros(2, device="cuda", dtype=torch.float64)
    small.train_step(xd[:4096], rd[:4096], stats=stats)  # loads the kernels' code before the measurement
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    f.train_step(xd, rd, stats=stats)
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    f.check_errors()
    s = stats.cpu().numpy()
    assert np.all(np.isfinite(s)) and s[1] > 0
    n_params = f.n_params
    b = f.device_bytes
    print(f"fused BF16 at 2^20: {b / 2**20:.1f} MiB held ({b / n_params:.1f} B/parameter), "
          f"allocated by creating two fields {(free0 - free1) / 2**20:.1f} MiB, "
          f"during the step {(free1 - free2) / 2**20:.1f} MiB")
    assert b == small.device_bytes                 # independent of max_batch
    assert b <= 28 * n_params + (8 << 20)          # w, w_inf, grad, m, v, steps, two 16-bit copies
    assert free2 == free1                          # the step allocates nothing
    f32 = nmg.GuidingField(nmg.config(1, path=nmg.PATH_FP32), max_queries=0, max_batch=N)
    b32 = f32.device_bytes
    per_record = (b32 - f32.n_params * 24) / N
    print(f"plain FP32 at 2^20: {b32 / 2**20:.1f} MiB ({per_record:.0f} B of stored activations per record)")
    assert b32 > b + N * 1500
    for g in (f, small, f32):
        g.close()
