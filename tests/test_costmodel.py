"""Host-side checks of the tuner and the learned cost model: candidate
enumeration, the separable feature vector, the MLP oracle's gradients
against finite differences, and the regret bookkeeping.  When the packaged
model and its timing set exist, the model must choose better plans than
the analytic planner on the held-out matrices."""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import costmodel, synthetic, tuning
from oracle import mlp as mlp_oracle


def test_candidates_cross_product():
    cands, nr, npp = tuning.candidates(8219, 8219, length_policy=gb.GBSP_LEN_7SMOOTH)
    assert nr == 8 and npp == 8 and len(cands) == 64  # every shape fits 8219 rows
    for i in range(nr):
        for j in range(npp):
            c = cands[i * npp + j]
            assert c.pass1_shape == cands[j].pass1_shape
            assert c.radices() == cands[i * npp].radices() and c.rows_threads == cands[i * npp].rows_threads
            assert int(np.prod(c.radices())) == 16464
    # the first candidate is the analytic planner's own choice
    with pytest.raises(gb.GbspError):
        tuning.candidates(8219, 8219, length_policy=gb.GBSP_LEN_7SMOOTH, pass1_shape=9)


def test_candidates_large_rows_prefer_two_level_table():
    # 40421 rows: neither a full nor a half table fits beside 256-row items;
    # the two-level table does (measured faster than 128-row items with the
    # half table), the half-table and two-level 128-row shapes follow
    cands, nr, npp = tuning.candidates(40421, 40421, length_policy=gb.GBSP_LEN_7SMOOTH)
    assert npp == 3 and [c.pass1_shape for c in cands[:3]] == [7, 6, 8]
    assert all(int(np.prod(c.radices())) * 3 == 81000 for c in cands)  # three channels of 27000


def test_features_are_separable():
    coo = synthetic.uniform_matrix(777, 1500, 9000, seed=3)
    cands, nr, npp = tuning.candidates(coo.rows, coo.cols, length_policy=gb.GBSP_LEN_7SMOOTH)
    F = np.array([tuning.features(coo, c) for c in cands]).reshape(nr, npp, -1)
    assert F.shape[2] == gb._capi.GBSP_N_FEATURES
    for i in range(nr):
        for j in range(npp):
            np.testing.assert_array_equal(F[i, j, tuning.F_MATRIX], F[0, 0, tuning.F_MATRIX])
            np.testing.assert_array_equal(F[i, j, tuning.F_ROWS], F[i, 0, tuning.F_ROWS])
            np.testing.assert_array_equal(F[i, j, tuning.F_PASS1], F[0, j, tuning.F_PASS1])
    assert F[0, 0, 0] == pytest.approx(np.log2(777))
    assert F[0, 0, 8] == 1.0  # one channel
    hist = F[0, 0, 10:16]
    assert hist.sum() == pytest.approx(1.0, abs=1e-6)


def test_oracle_gradient_matches_finite_differences():
    g = np.random.default_rng(0)
    n_in = 7
    p = costmodel.init_params(n_in, seed=1).astype(np.float64)
    x = g.normal(size=(40, n_in))
    t = g.normal(size=40)
    _, grad = mlp_oracle.loss_and_grad(p, x, t)
    h = 1e-6
    for k in g.choice(p.size, 60, replace=False):
        e = np.zeros_like(p)
        e[k] = h
        num = (mlp_oracle.loss_and_grad(p + e, x, t)[0] - mlp_oracle.loss_and_grad(p - e, x, t)[0]) / (2 * h)
        assert grad[k] == pytest.approx(num, rel=1e-4, abs=1e-8)


def test_param_count_matches_layout():
    n = costmodel.param_count(36)
    assert n == 36 * 64 + 64 + 64 * 64 + 64 + 64 + 1
    assert costmodel.init_params(36).size == n


def fake_dataset():
    g = np.random.default_rng(5)
    N = 6
    ds = {"M": g.normal(size=(N, 18)).astype(np.float32), "R": g.normal(size=(N, 8, 10)).astype(np.float32),
          "P": g.normal(size=(N, 6, 8)).astype(np.float32),
          "ms_rows": np.full((N, 8), np.nan, np.float32), "ms_pass1": np.full((N, 6), np.nan, np.float32),
          "n_rows": np.array([8, 3, 5, 8, 1, 2], np.int32), "n_p1": np.array([6, 1, 6, 2, 1, 6], np.int32),
          "n_test": np.int32(2)}
    for k in range(N):
        ds["ms_rows"][k, :ds["n_rows"][k]] = g.uniform(0.1, 1.0, ds["n_rows"][k])
        ds["ms_pass1"][k, :ds["n_p1"][k]] = g.uniform(0.1, 1.0, ds["n_p1"][k])
    return ds


def test_compose_and_regret():
    ds = fake_dataset()
    X, y, gid = costmodel.compose(ds, range(6))
    assert X.shape == (int((ds["n_rows"] * ds["n_p1"]).sum()), 36)
    # an oracle score (the true log time) has zero regret; the analytic choice (0, 0) has its own
    r = costmodel.regret(ds, range(6), y)
    assert r["max"] == pytest.approx(0.0, abs=1e-6)
    r0 = costmodel.regret(ds, range(6))
    t = ds["ms_rows"][0, :8, None] + ds["ms_pass1"][0, None, :6]
    assert r0["max"] >= t[0, 0] / t.min() - 1 - 1e-6
    tr, te = costmodel.split(ds)
    assert list(tr) == [0, 1, 2, 3] and list(te) == [4, 5]


@pytest.mark.skipif(not costmodel.DEFAULT_MODEL.exists() or not costmodel.DEFAULT_DATA.exists(),
                    reason="packaged cost model not trained yet")
def test_packaged_model_domain():
    # the stored range is that of the training candidates: every held-out
    # matrix of the same generator lies inside it, the 40421 x 40421
    # adjacency (three channels, rows far above 12000) does not
    ds = costmodel.load_dataset()
    model = costmodel.load_model()
    tr, te = costmodel.split(ds)
    X, _, _ = costmodel.compose(ds, tr)
    np.testing.assert_array_equal(model["lo"], X.min(0))
    np.testing.assert_array_equal(model["hi"], X.max(0))
    for k in te[:50]:
        Xk, _, _ = costmodel.compose(ds, [k])
        assert costmodel.in_domain(model, Xk)
    coo = synthetic.config_matrix("uniform_powerlaw_40421")
    cands, _, _ = tuning.candidates(coo.rows, coo.cols, length_policy=gb.GBSP_LEN_7SMOOTH, index_bytes=4)
    assert not costmodel.in_domain(model, np.array([tuning.features(coo, c) for c in cands]))


@pytest.mark.skipif(not costmodel.DEFAULT_MODEL.exists() or not costmodel.DEFAULT_DATA.exists(),
                    reason="packaged cost model not trained yet")
def test_packaged_model_beats_analytic_planner():
    ds = costmodel.load_dataset()
    model = costmodel.load_model()
    _, te = costmodel.split(ds)
    X, _, _ = costmodel.compose(ds, te)
    pred = mlp_oracle.forward(model["params"], (X - model["mean"]) / model["scale"])
    learned = costmodel.regret(ds, te, pred)
    analytic = costmodel.regret(ds, te)
    assert learned["mean"] < analytic["mean"], (learned, analytic)
