"""GPU checks of the learned cost model and the autotuner.

The training and inference kernels (gbsp_mlp_forward / _backward / _adam)
against the float64 oracle in oracle/mlp.py, their determinism, a training
run that must fit, the exhaustive autotuner's bookkeeping, and plans made
by the learned planner (same spectrum as any other plan)."""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import costmodel, synthetic, tuning
from oracle import fp64
from oracle import mlp as mlp_oracle

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.tensor(np.asarray(a, np.float32), device="cuda")


@pytest.mark.parametrize("n", [1, 15, 16, 17, 1000, 5003])
def test_forward_matches_oracle(cuda, n):
    g = np.random.default_rng(n)
    p = costmodel.init_params(36, seed=n)
    x = g.normal(size=(n, 36)).astype(np.float32)
    net = costmodel.MLP(p)
    y = net.forward(dev(x)).cpu().numpy()
    ref = mlp_oracle.forward(p, x)
    np.testing.assert_allclose(y, ref, rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("n", [3, 16, 4099])
def test_backward_matches_oracle(cuda, n):
    g = np.random.default_rng(100 + n)
    p = costmodel.init_params(36, seed=2)
    x = g.normal(size=(n, 36)).astype(np.float32)
    t = g.normal(size=n).astype(np.float32)
    net = costmodel.MLP(p)
    net.backward(dev(x), dev(t))
    grad = net.g.cpu().numpy()
    loss = float(net.loss.item())
    ref_loss, ref_grad = mlp_oracle.loss_and_grad(p, x, t)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    err = np.linalg.norm(grad - ref_grad) / np.linalg.norm(ref_grad)
    assert err < 1e-4, err
    # fixed reduction order: bit-identical on a second run
    g1 = net.g.clone()
    net.backward(dev(x), dev(t))
    assert bool((net.g == g1).all())


def test_adam_matches_oracle(cuda):
    g = np.random.default_rng(3)
    p = costmodel.init_params(36, seed=3)
    net = costmodel.MLP(p)
    pr, m, v = p.astype(np.float64), np.zeros(p.size), np.zeros(p.size)
    for step in range(1, 4):
        grad = g.normal(size=p.size).astype(np.float32)
        net.g.copy_(dev(grad))
        net.adam(1e-3)
        pr, m, v = mlp_oracle.adam(pr, grad.astype(np.float64), m, v, 1e-3, 0.9, 0.999, 1e-8, step)
    np.testing.assert_allclose(net.params(), pr, rtol=1e-5, atol=1e-6)


def test_training_fits_a_smooth_target(cuda):
    g = np.random.default_rng(4)
    x = g.normal(size=(4096, 36)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.3 * np.abs(x[:, 3])).astype(np.float32)
    net = costmodel.MLP(costmodel.init_params(36, seed=4))
    xd, td = dev(x), dev(t)
    net.backward(xd, td)
    first = float(net.loss.item())
    for _ in range(400):
        net.backward(xd, td)
        net.adam(3e-3)
    net.backward(xd, td)
    assert float(net.loss.item()) < 0.1 * first


def test_autotune_small_matrix(cuda):
    import torch
    coo = synthetic.uniform_matrix(601, 900, 6000, seed=8)
    tr = tuning.autotune(coo, reps=2, length_policy=gb.GBSP_LEN_7SMOOTH)
    assert tr.n_rows >= 2 and tr.n_p1 >= 2
    assert np.all(np.isfinite(tr.ms_rows)) and np.all(np.isfinite(tr.ms_pass1))
    tot = tr.total()
    i, j = np.unravel_index(np.argmin(tot), tot.shape)
    assert tr.best.radices() == tr.candidates[i * tr.n_p1 + j].radices()
    assert tr.best.pass1_shape == tr.candidates[i * tr.n_p1 + j].pass1_shape
    half = coo.rows // 2 + 1
    assert tr.best.u_tile in (0, half // 2, half // 4)
    with gb.Plan(coo, options=tr.best) as plan:
        out = plan.empty_output()
        plan.execute(out)
        torch.cuda.synchronize()
        assert plan.info["pass1_shape"] == tr.best.pass1_shape
        got = out.cpu().numpy()[:, :coo.cols // 2 + 1]
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got, ref) < 1e-5


def test_autotune_tile_respects_the_callers_limit(cuda):
    coo = synthetic.uniform_matrix(601, 900, 6000, seed=8)
    tr = tuning.autotune(coo, reps=1, max_rows_cands=2, u_tile=128)
    assert tr.best.u_tile in (128, 64, 32)
    assert all(c.u_tile == 128 for c in tr.candidates)


def test_learned_planner_picks_the_predicted_best(cuda):
    import torch
    model = costmodel.load_model() if costmodel.DEFAULT_MODEL.exists() else {
        "params": costmodel.init_params(36, seed=9), "mean": np.zeros(36, np.float32),
        "scale": np.ones(36, np.float32)}
    costmodel.install(model)
    costmodel._installed = True  # planner="learned" uses the model just installed
    coo = synthetic.uniform_matrix(1201, 2500, 20000, seed=10)
    cands, nr, npp = tuning.candidates(coo.rows, coo.cols, length_policy=gb.GBSP_LEN_7SMOOTH)
    X = np.array([tuning.features(coo, c) for c in cands])
    pred = costmodel.predict(model, X)
    want = cands[int(np.argmin(pred))]
    with gb.Plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, planner="learned") as plan:
        info = plan.info
        assert info["planner"] == gb._capi.GBSP_PLANNER_LEARNED
        assert tuple(info["radix"]) == want.radices()
        assert info["rows_threads"] == want.rows_threads and info["pass1_shape"] == want.pass1_shape
        out = plan.empty_output()
        plan.execute(out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()[:, :coo.cols // 2 + 1]
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got, ref) < 1e-5


def test_learned_planner_outside_its_domain(cuda):
    # a matrix whose candidates leave the training range (16706 columns: two
    # channels, which the batch generator never produces) keeps the analytic
    # choice; clearing the range lets the network decide
    if not costmodel.DEFAULT_MODEL.exists():
        pytest.skip("packaged cost model not trained yet")
    model = costmodel.load_model()
    assert "lo" in model
    costmodel.install(model)
    costmodel._installed = True
    coo = synthetic.uniform_matrix(2001, 16706, 30000, seed=11)
    cands, nr, npp = tuning.candidates(coo.rows, coo.cols, length_policy=gb.GBSP_LEN_7SMOOTH)
    X = np.array([tuning.features(coo, c) for c in cands])
    assert not costmodel.in_domain(model, X)
    with gb.Plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, planner="learned") as plan:
        assert plan.info["planner"] == gb._capi.GBSP_PLANNER_MODEL
        assert tuple(plan.info["radix"]) == cands[0].radices()
        assert plan.info["pass1_shape"] == cands[0].pass1_shape
    lib = gb._capi.load()
    gb._capi.check(lib.gbsp_cost_model_set_domain(0, None, None), "gbsp_cost_model_set_domain")
    try:
        want = cands[int(np.argmin(costmodel.predict(model, X)))]
        with gb.Plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, planner="learned") as plan:
            assert plan.info["planner"] == gb._capi.GBSP_PLANNER_LEARNED
            assert tuple(plan.info["radix"]) == want.radices()
    finally:
        costmodel.install(model)


def test_learned_batch(cuda):
    import torch
    if not costmodel.DEFAULT_MODEL.exists():
        pytest.skip("packaged cost model not trained yet")
    mats = synthetic.batch_matrices(64)[:6]
    with gb.Batch(mats, length_policy=gb.GBSP_LEN_7SMOOTH, planner="learned") as b:
        outs = b.empty_outputs()
        b.set_outputs(outs)
        b.graph_launch()
        torch.cuda.synchronize()
        assert all(i["planner"] == gb._capi.GBSP_PLANNER_LEARNED for i in b.infos)
        for coo, o in zip(mats[:2], outs):
            us = np.array([0, 1, coo.rows // 2, coo.rows - 1])
            ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
            assert fp64.rel_l2(o.cpu().numpy()[us, :coo.cols // 2 + 1], ref) < 1e-5
