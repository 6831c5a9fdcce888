"""nmg_mixture_loss_grad_noalloc: the loss/gradient entry point for callers
that cannot allocate device memory (every byte pooled before the frame loop,
no allocator of their own, or no room for the synchronisation an allocation
can cause). It must give the results of nmg_mixture_loss_grad, which reduces
the FP64 loss sum through a caller-provided workspace, while allocating
nothing itself: its block sums live in a fixed array inside libnmg.so.

Called through the C ABI. Two calls in a row (with different batch sizes, so
stale contents of the shared array would show), each compared with the
workspace entry point: gradients and per-sample losses bit-identical (same
per-sample kernel), the FP64 loss sum equal to 1e-12 relative (its additions
are grouped differently).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    P = ctypes.c_void_p
    lib.nmg_mixture_loss_grad_noalloc.argtypes = [ctypes.c_void_p, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                  P, P, P, P]
    lib.nmg_mixture_loss_grad_noalloc.restype = ctypes.c_int


def _noalloc(nmg, raw, rec, K, selection=False):
    import torch
    lib = nmg.lib()
    _bind(lib)
    n = raw.shape[0]
    g = torch.zeros_like(raw)
    loss = torch.empty(n, device="cuda")
    tot = torch.full((1,), -1.0, device="cuda", dtype=torch.float64)
    o = nmg.mixture_opts(K, raw.shape[1], selection=selection)
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.nmg_mixture_loss_grad_noalloc(ctypes.byref(o), raw.data_ptr(), rec.data_ptr(), rec.shape[1], n, 128.0,
                                           g.data_ptr(), loss.data_ptr(), tot.data_ptr(), ctypes.c_void_p(st))
    return rc, g, loss, tot


def test_noalloc_matches_workspace_entry_point(nmg, synth):
    import torch
    for n, K, sel in ((65536, 8, False), (1000, 7, True)):
        raw, _, rec = synth.mixture_batch(n, K, seed=n, selection=sel)
        r, rc = torch.from_numpy(raw).cuda(), torch.from_numpy(rec).cuda()
        g_ref, l_ref, t_ref = nmg.mixture_loss_grad(r, rc, K, 128.0, selection=sel)
        status, g, loss, tot = _noalloc(nmg, r, rc, K, sel)
        torch.cuda.synchronize()
        assert status == 0, nmg.lib().nmg_last_error()
        assert torch.equal(g, g_ref)
        assert torch.equal(loss, l_ref)
        a, b = float(tot.cpu()[0]), float(t_ref.cpu()[0])
        assert abs(a - b) <= 1e-12 * abs(b)


def test_noalloc_rejects_oversize_batch(nmg):
    lib = nmg.lib()
    _bind(lib)
    o = nmg.mixture_opts(8, 32)
    rc = lib.nmg_mixture_loss_grad_noalloc(ctypes.byref(o), None, None, 6, 1048577, 128.0, None, None, None, None)
    assert rc == 7  # NMG_ERR_CAPACITY, checked on the host before any device work
    assert b"1048576" in lib.nmg_last_error()
