"""Plan memory: each plan's device memory is one allocation from a
stream-ordered pool private to the library, which keeps freed memory (up to
gbsp_set_memory_cache's limit) for later plans.  Reused memory must give
bit-identical spectra, whatever the limit and however plans overlap."""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import synthetic
from oracle import fp64

pytestmark = pytest.mark.gpu

DEFAULT_CACHE = 1 << 30


def spectrum(plan):
    import torch
    out = plan.empty_output()
    out.fill_(complex(3.0, 3.0))
    plan.execute(out)
    torch.cuda.synchronize()
    assert plan.error_flags() == 0
    return out.cpu().numpy()


def test_reused_plan_memory_gives_identical_spectra(cuda):
    coo = synthetic.uniform_matrix(1201, 2500, 20000, seed=3)
    got = []
    try:
        for limit in (DEFAULT_CACHE, 0, DEFAULT_CACHE, 1 << 20):
            gb.set_memory_cache(limit)
            for _ in range(2):
                with gb.Plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH) as p:
                    got.append(spectrum(p))
    finally:
        gb.set_memory_cache(DEFAULT_CACHE)
    assert all(np.array_equal(got[0], g) for g in got[1:])
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got[0][:, :coo.cols // 2 + 1], ref) <= 1e-5


def test_overlapping_plans(cuda):
    # plans alive together and destroyed out of order never share memory
    a = synthetic.uniform_matrix(700, 900, 9000, seed=4)
    b = synthetic.uniform_matrix(1500, 333, 12000, seed=5)
    pa = gb.Plan(a)
    pb = gb.Plan(b)
    want_a, want_b = spectrum(pa), spectrum(pb)
    pa.close()
    pc = gb.Plan(a)  # likely reuses pa's memory while pb is alive
    assert np.array_equal(spectrum(pb), want_b)
    assert np.array_equal(spectrum(pc), want_a)
    pb.close()
    pc.close()


def test_pass1_item_queue_rearms(cuda):
    # pass 1 hands out work items from a device counter that the last CTA of
    # each launch zeroes again: repeated and interleaved launches of two
    # plans (whole transforms, tiles, pass 1 alone) must all see a fresh queue
    import torch
    a = synthetic.uniform_matrix(900, 700, 12000, seed=6)
    b = synthetic.uniform_matrix(333, 1500, 8000, seed=7)
    with gb.Plan(a) as pa, gb.Plan(b, u_tile=40) as pb:
        want_a, want_b = spectrum(pa), spectrum(pb)
        for _ in range(3):
            s = torch.zeros((50, 704), dtype=torch.complex64, device="cuda")
            pa.column_sums(10, 50, s)
            assert np.array_equal(spectrum(pb), want_b)
            assert np.array_equal(spectrum(pa), want_a)
