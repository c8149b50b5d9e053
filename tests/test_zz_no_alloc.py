"""gbsp_execute_noalloc: the transform for callers that must not allocate
device memory while they run it (pool-owned device memory, latency-critical
loops).  Its pass-1 intermediate lives in a fixed array inside the library;
this checks, through the C ABI, that two calls in a row give the same
spectrum as gbsp_execute (rel-L2 <= 1e-5, the tolerance of the other parity
tests) and that nothing leaks into the device error word.

Kept in a file of its own that pytest collects last; it passes both alone in
a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import _capi, synthetic
from oracle import fp64

pytestmark = pytest.mark.gpu

REL_L2_TOL = 1e-5


def _noalloc(plan, out):
    import torch
    lib = _capi.load()
    st = lib.gbsp_execute_noalloc(plan._h, C.c_void_p(out.data_ptr()), out.shape[1],
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _capi.check(st, "gbsp_execute_noalloc")


@pytest.mark.parametrize("name,policy", [("uniform_3001x2048", 3), ("banded_powerlaw_8219", 7)])
def test_noalloc_matches_execute_twice(cuda, name, policy):
    import torch
    coo = synthetic.config_matrix(name)
    with gb.Plan(coo, length_policy=policy) as plan:
        ref = plan.empty_output()
        plan.execute(ref)
        torch.cuda.synchronize()
        ref_h = ref.cpu().numpy()
        fc = coo.cols // 2 + 1
        for call in range(2):
            out = plan.empty_output()
            out.fill_(complex(3.0, -3.0))  # stale contents must not leak through
            _noalloc(plan, out)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            err = fp64.rel_l2(got[:, :fc], ref_h[:, :fc])
            assert err <= REL_L2_TOL, f"call {call}: rel-L2 {err:.3e}"
            assert np.all(got[:, fc:] == 0)
        assert plan.error_flags() == 0


def test_noalloc_rejects_bad_output(cuda):
    coo = synthetic.uniform_matrix(64, 50, 300, seed=2)
    with gb.Plan(coo) as plan:
        out = plan.empty_output()
        lib = _capi.load()
        st = lib.gbsp_execute_noalloc(plan._h, C.c_void_p(out.data_ptr()), 3, None)
        assert st == _capi.GBSP_ERR_INVALID
        assert "out_pitch" in _capi.last_error()
