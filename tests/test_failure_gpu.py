"""Failure detection without a GPU fault (include/nmg.h: nmg_selftest_wait_timeout).

Every device-side wait in the fused kernels is bounded: when one gives up, the kernel records a
code in the context's device error flag and returns, and nmg_check_errors reports
NMG_ERR_TIMEOUT. The self-test kernel waits, through that same bounded wait, on a barrier that
nothing arrives at, so the wait runs out by its own limit (about a second at the maximum SM
clock); nothing traps or faults. The test checks the status the host reads and that the context
keeps working afterwards.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NMG_ERR_TIMEOUT, NMG_ERR_UNSUPPORTED = 5, 6


def test_bounded_wait_timeout_is_reported_and_the_context_recovers(nmg, synth):
    import torch
    f = nmg.GuidingField(nmg.config(nmg.PRESET_HASHGRID, path=nmg.PATH_BF16), max_queries=4096, max_batch=4096)
    try:
        q = synth.wavefront(4096, seed=3)
        dq = [torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("pos", "wo", "normal", "rough", "u4")]
        ref = f.query(*dq)
        f.check_errors()
        t0 = time.perf_counter()
        f.selftest_wait_timeout()
        with pytest.raises(nmg.NMGError) as e:
            f.check_errors()
        waited = time.perf_counter() - t0
        assert e.value.status == NMG_ERR_TIMEOUT
        assert b"code 9" in nmg.lib().nmg_last_error()
        assert 0.2 < waited < 30.0, waited  # the wait ran to its limit, and the limit ended it
        f.check_errors()  # reading the error cleared the flag
        out = f.query(*dq)  # the same context still answers, with the same results
        torch.cuda.synchronize()
        assert torch.equal(out["dir"], ref["dir"]) and torch.equal(out["pdf"], ref["pdf"])
        f.check_errors()
    finally:
        f.close()


def test_selftest_needs_fused_kernel_state(nmg):
    f = nmg.GuidingField(nmg.config(path=nmg.PATH_FP32))
    try:
        with pytest.raises(nmg.NMGError) as e:
            f.selftest_wait_timeout()
        assert e.value.status == NMG_ERR_UNSUPPORTED
    finally:
        f.close()
