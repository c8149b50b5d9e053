"""Batched transforms (gbsp_batch_*): one persistent launch per pass over
many matrices of uneven size and sparsity, fed by device work queues.

Every batched output must be bit-identical to the single-matrix plan built
with the same kernel configuration (same pass-1 shape, radices, block size
and index width), and within rel-L2 1e-5 of the FP64 oracle.  Matrices whose
convolution is split into clusters run through their own plan inside the
batch; they are checked the same way.
"""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import synthetic
from oracle import fp64

pytestmark = pytest.mark.gpu

REL_L2_TOL = 1e-5


def mixed_batch(count, seed, lo=5, hi=700):
    g = np.random.default_rng(seed)
    mats = []
    for i in range(count):
        r = int(g.integers(lo, hi))
        c = int(g.integers(lo, hi))
        dens = float(np.exp(g.uniform(np.log(2e-3), np.log(5e-2))))
        mats.append(synthetic.uniform_matrix(r, c, max(1, int(r * c * dens)), seed * 1000 + i))
    # edge shapes: one row, one column, an empty matrix, a dense corner
    mats.append(synthetic.uniform_matrix(1, 37, 9, seed + 1))
    mats.append(synthetic.uniform_matrix(41, 1, 9, seed + 2))
    mats.append(gb.COOMatrix(19, 23, np.zeros(0, np.int32), np.zeros(0, np.int32)))
    mats.append(synthetic.uniform_matrix(16, 16, 400, seed + 3))
    return mats


def single_plan_output(coo, info, **kw):
    import torch
    radix = info["radix"] if info["channels"] == 1 else None
    with gb.Plan(coo, rows_threads=info["rows_threads"] if info["channels"] == 1 else 0, radix=radix,
                 index_bytes=info["index_bytes"], row_table_mode=1 + info["row_table_mode"], **kw) as plan:
        out = plan.empty_output()
        plan.execute(out)
        torch.cuda.synchronize()
        return out.cpu().numpy()


def run_batch(mats, graph=False, repeats=1, **kw):
    import torch
    with gb.Batch(mats, **kw) as b:
        outs = b.empty_outputs()
        for o in outs:
            o.fill_(complex(7.0, 7.0))  # poison: every element must be overwritten
        b.set_outputs(outs)
        for _ in range(repeats):
            (b.graph_launch if graph else b.execute)()
        torch.cuda.synchronize()
        assert b.error_flags() == 0
        return [o.cpu().numpy() for o in outs], b.infos


def check_oracle(coo, got):
    fc = coo.cols // 2 + 1
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    err = fp64.rel_l2(got[:, :fc], ref) if np.abs(ref).max() > 0 else float(np.abs(got[:, :fc]).max())
    assert err <= REL_L2_TOL, f"{coo.rows}x{coo.cols}: rel-L2 {err:.3e}"
    assert np.all(got[:, fc:] == 0)


@pytest.mark.parametrize("policy", [gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH])
def test_batch_matches_single_plans(cuda, policy):
    mats = mixed_batch(24, seed=11 + policy)
    outs, infos = run_batch(mats, length_policy=policy)
    for coo, got, info in zip(mats, outs, infos):
        assert info["rows_threads"] in (256, 512) and info["channels"] == 1
        want = single_plan_output(coo, info, length_policy=policy)
        assert np.array_equal(got, want), f"{coo.rows}x{coo.cols} differs from its single plan"
        check_oracle(coo, got)


def test_batch_with_cluster_matrices(cuda):
    # max_channel_len 400 splits every convolution longer than 400 into channels
    mats = mixed_batch(10, seed=5, lo=100, hi=900)
    outs, infos = run_batch(mats, length_policy=gb.GBSP_LEN_7SMOOTH, max_channel_len=400)
    assert any(i["channels"] > 1 for i in infos) and any(i["channels"] == 1 for i in infos)
    for coo, got in zip(mats, outs):
        check_oracle(coo, got)


def test_batch_graph_and_repeats(cuda):
    mats = mixed_batch(12, seed=23)
    once, _ = run_batch(mats, length_policy=gb.GBSP_LEN_7SMOOTH)
    replay, _ = run_batch(mats, graph=True, repeats=3, length_policy=gb.GBSP_LEN_7SMOOTH)
    again, _ = run_batch(mats, repeats=4, length_policy=gb.GBSP_LEN_7SMOOTH)
    for a, b, c in zip(once, replay, again):
        assert np.array_equal(a, b) and np.array_equal(a, c)


def test_batch_rebind_outputs(cuda):
    import torch
    mats = mixed_batch(6, seed=31)
    with gb.Batch(mats, length_policy=gb.GBSP_LEN_3SMOOTH) as b:
        first = b.empty_outputs()
        b.set_outputs(first)
        b.graph_launch()
        second = [torch.full_like(o, complex(3.0, 3.0)) for o in first]
        b.set_outputs(second)  # the graph is captured again for the new pointers
        b.graph_launch()
        torch.cuda.synchronize()
        for x, y in zip(first, second):
            assert torch.equal(x, y)


def test_batch_of_benchmark_generator(cuda):
    # eight matrices of the 64-matrix batched workload (dims in [500, 12000])
    mats = synthetic.batch_matrices(64)[:8]
    outs, infos = run_batch(mats, length_policy=gb.GBSP_LEN_7SMOOTH)
    for coo, got, info in zip(mats[:3], outs, infos):
        us = np.unique(np.r_[0:3, coo.rows // 2 - 1:coo.rows // 2 + 2, coo.rows - 3:coo.rows] % coo.rows)
        ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
        assert fp64.rel_l2(got[us, :coo.cols // 2 + 1], ref) <= REL_L2_TOL


def test_batch_rejects_bad_outputs(cuda):
    import torch
    mats = mixed_batch(2, seed=3)
    with gb.Batch(mats) as b:
        with pytest.raises(gb.GbspError):
            b.execute()  # outputs not bound
        outs = b.empty_outputs()
        bad = [torch.empty((o.shape[0], 1), dtype=torch.complex64, device="cuda") for o in outs]
        with pytest.raises(gb.GbspError):
            b.set_outputs(bad)
