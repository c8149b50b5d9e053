"""gbsp_execute_noalloc: the transform for callers that must not allocate
device memory while they run it (pool-owned device memory, latency-critical
loops).  Its pass-1 intermediate lives in a fixed array inside the library;
this checks, through the C ABI, that two calls in a row give the same
spectrum as gbsp_execute (rel-L2 <= 1e-5, the tolerance of the other parity
tests), that each call is within 1e-5 of the FP64 oracle, and that nothing
leaks into the device error word.  The shapes cover one tile and many tiles
of the array, and the single-channel, sequential-channel (two channels) and
wide sequential-channel (more than eight channels) row kernels.

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


SCRATCH_BYTES = 32 << 20  # the library's fixed array


def noalloc_tiles(info, cols):
    """Tiles of Bluestein rows one call runs: rows of the pass-1 intermediate
    (columns rounded up to even, pitch to 16) that fit the array."""
    s_pitch = ((cols + 1) // 2 * 2 + 15) // 16 * 16
    tile = min(info["u_tile"], SCRATCH_BYTES // (s_pitch * 8))
    return -(-info["half_rows"] // tile)


def wide_matrix():
    g = np.random.default_rng(120001)
    rows, cols, n = 300, 120001, 480_000
    return synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))


CASES = [("uniform_3001x2048", 3, 1, None), ("banded_powerlaw_8219", 7, 9, 0),
         ("uniform_powerlaw_16706", 7, 34, 2), ("wide_300x120001", 7, 5, 2)]


@pytest.mark.parametrize("name,policy,tiles,channel_mode", CASES)
def test_noalloc_matches_execute_twice(cuda, name, policy, tiles, channel_mode):
    import torch
    coo = wide_matrix() if name.startswith("wide") else synthetic.config_matrix(name)
    with gb.Plan(coo, length_policy=policy) as plan:
        info = plan.info
        assert noalloc_tiles(info, coo.cols) == tiles
        if channel_mode is not None:
            assert info["channel_mode"] == channel_mode
        ref = plan.empty_output()
        plan.execute(ref)
        torch.cuda.synchronize()
        ref_h = ref.cpu().numpy()
        fc = coo.cols // 2 + 1
        small = coo.rows * coo.cols <= 3001 * 2048
        us = None if small else np.unique(np.r_[0, 1, 255, 256, 511, coo.rows // 2, coo.rows - 1,
                                                np.random.default_rng(1).integers(0, coo.rows, 6)] % coo.rows)
        exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
        for call in range(2):
            out = plan.empty_output()
            out.fill_(complex(3.0, -3.0))  # stale contents must not leak through
            _noalloc(plan, out)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            err = fp64.rel_l2(got[:, :fc], ref_h[:, :fc])
            assert err <= REL_L2_TOL, f"call {call}: rel-L2 {err:.3e} vs gbsp_execute"
            sub = got[:, :fc] if us is None else got[us, :fc]
            err = fp64.rel_l2(sub, exact)
            assert err <= REL_L2_TOL, f"call {call}: rel-L2 {err:.3e} vs FP64"
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
