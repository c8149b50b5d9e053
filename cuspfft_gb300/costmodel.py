"""Learned cost model: an MLP (36 features -> 64 -> 64 -> log ms) trained on
the autotuner's own timings, predicting each candidate's latency so a plan
can be chosen without measuring (planner="learned").

Everything numeric runs in the library's hand-written kernels
(gbsp_mlp_forward / gbsp_mlp_backward / gbsp_mlp_adam); torch only provides
device memory.  The exhaustive autotuner stays the fallback and the arbiter of
the model's regret.  The spectrum never depends on the model.

Dataset (one row per matrix, padded to 8 row choices x 6 pass-1 shapes):
  M [N, 18]      matrix features          R [N, 8, 10]   row-choice features
  P [N, 6, 8]    pass-1 shape features    ms_rows [N, 8], ms_pass1 [N, 6]
  n_rows, n_p1 [N], dims [N, 3] (rows, cols, nnz)
The feature of candidate (i, j) is concat(M, R[i], P[j]) (gbsp_plan_features
is separable this way) and its time ms_rows[i] + ms_pass1[j] (the phases are
timed separately).  Candidate (0, 0) is what the analytic planner builds.

Command line (needs a GPU):
  python -m cuspfft_gb300.costmodel collect --out tune.npz [--train 2000 --test 200]
  python -m cuspfft_gb300.costmodel train --data tune.npz --out model.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time
from pathlib import Path
from typing import Optional

import numpy as np

from ._capi import GBSP_LEN_7SMOOTH, GBSP_MLP_HIDDEN, GBSP_N_FEATURES, check, load
from . import synthetic, tuning

DATA_DIR = Path(__file__).resolve().parent / "data"
DEFAULT_MODEL = DATA_DIR / "cost_model.npz"
DEFAULT_DATA = DATA_DIR / "tune_timings.npz"
MAX_R, MAX_P = 8, 8
N_M, N_R, N_P = 18, 10, 8
H = GBSP_MLP_HIDDEN


def param_count(n_in: int = GBSP_N_FEATURES) -> int:
    return int(load().gbsp_mlp_param_count(n_in))


def init_params(n_in: int = GBSP_N_FEATURES, seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases, packed W1, b1, W2, b2, w3, b3."""
    g = np.random.default_rng(seed)
    w1 = g.normal(0, math.sqrt(2.0 / n_in), (n_in, H))
    w2 = g.normal(0, math.sqrt(2.0 / H), (H, H))
    w3 = g.normal(0, math.sqrt(1.0 / H), H)
    return np.concatenate([w1.ravel(), np.zeros(H), w2.ravel(), np.zeros(H), w3, [0.0]]).astype(np.float32)


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class MLP:
    """Device-resident network with the library's training kernels."""

    def __init__(self, params: np.ndarray, n_in: int = GBSP_N_FEATURES):
        import torch
        self.lib = load()
        self.n_in = n_in
        self.n_params = param_count(n_in)
        if params.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {params.size}")
        dev = torch.device("cuda")
        self.p = torch.tensor(params, dtype=torch.float32, device=dev)
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.loss = torch.zeros(1, dtype=torch.float32, device=dev)
        self.work = torch.zeros(int(self.lib.gbsp_mlp_work_floats(n_in)), dtype=torch.float32, device=dev)
        self.step_no = 0

    def forward(self, x) -> "torch.Tensor":
        import torch
        y = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        check(self.lib.gbsp_mlp_forward(_ptr(self.p), self.n_in, _ptr(x), x.shape[0], _ptr(y), None),
              "gbsp_mlp_forward")
        return y

    def backward(self, x, t) -> None:
        """self.g <- d mean((f(x) - t)^2) / d params; self.loss <- the loss."""
        check(self.lib.gbsp_mlp_backward(_ptr(self.p), self.n_in, _ptr(x), _ptr(t), x.shape[0], _ptr(self.g),
                                         _ptr(self.loss), _ptr(self.work), None), "gbsp_mlp_backward")

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step_no += 1
        check(self.lib.gbsp_mlp_adam(_ptr(self.p), _ptr(self.g), _ptr(self.m), _ptr(self.v), self.n_params, lr,
                                     beta1, beta2, eps, self.step_no, None), "gbsp_mlp_adam")

    def params(self) -> np.ndarray:
        return self.p.cpu().numpy().copy()


# ---------------------------------------------------------------------------
# dataset
# ---------------------------------------------------------------------------
def dataset_matrices(n: int, seed: int):
    """Seeded matrices from the batched-workload generator (dims log-uniform
    in [500, 12000], half prime and half 5-smooth, density 1e-4..1e-2)."""
    for i, (r, c, d) in enumerate(synthetic.batch_dims(n, seed=seed)):
        yield synthetic.uniform_matrix(r, c, max(1, int(round(r * c * d))), seed * 100003 + i)


def collect(mats, policy: int = GBSP_LEN_7SMOOTH, reps: int = 3, log_every: int = 100, **opts) -> dict:
    N = len(mats)
    ds = {
        "M": np.zeros((N, N_M), np.float32), "R": np.zeros((N, MAX_R, N_R), np.float32),
        "P": np.zeros((N, MAX_P, N_P), np.float32), "ms_rows": np.full((N, MAX_R), np.nan, np.float32),
        "ms_pass1": np.full((N, MAX_P), np.nan, np.float32), "n_rows": np.zeros(N, np.int32),
        "n_p1": np.zeros(N, np.int32), "dims": np.zeros((N, 3), np.int64),
        "policy": np.int32(policy),
    }
    from .sparse_fft import make_compact_csc
    t0 = time.time()
    for k, coo in enumerate(mats):
        csc = make_compact_csc(coo)
        tr = tuning.autotune(coo, csc=csc, reps=reps, length_policy=policy, **opts)
        ds["n_rows"][k], ds["n_p1"][k] = tr.n_rows, tr.n_p1
        ds["dims"][k] = (coo.rows, coo.cols, coo.nnz)
        ds["ms_rows"][k, :tr.n_rows] = tr.ms_rows
        ds["ms_pass1"][k, :tr.n_p1] = tr.ms_pass1
        for i in range(tr.n_rows):
            f = tuning.features(coo, tr.candidates[i * tr.n_p1], csc=csc)
            ds["R"][k, i] = f[tuning.F_ROWS]
            if i == 0:
                ds["M"][k] = f[tuning.F_MATRIX]
        for j in range(tr.n_p1):
            ds["P"][k, j] = tuning.features(coo, tr.candidates[j], csc=csc)[tuning.F_PASS1]
        if log_every and (k + 1) % log_every == 0:
            print(f"collect: {k + 1}/{N} matrices, {time.time() - t0:.0f} s", flush=True)
    return ds


def compose(ds: dict, idx) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(X, log ms, matrix id) over every candidate of the matrices in idx."""
    X, y, gid = [], [], []
    for k in idx:
        nr, npp = int(ds["n_rows"][k]), int(ds["n_p1"][k])
        for i in range(nr):
            for j in range(npp):
                X.append(np.concatenate([ds["M"][k], ds["R"][k, i], ds["P"][k, j]]))
                y.append(math.log(float(ds["ms_rows"][k, i]) + float(ds["ms_pass1"][k, j])))
                gid.append(k)
    return np.asarray(X, np.float32), np.asarray(y, np.float32), np.asarray(gid, np.int64)


def regret(ds: dict, idx, scores: Optional[np.ndarray] = None) -> dict:
    """Regret (time of the chosen candidate / exhaustive best - 1) over the
    matrices in idx.  scores: predicted log ms in compose() order (None =
    the analytic planner's choice, candidate (0, 0))."""
    out, pos = [], 0
    for k in idx:
        nr, npp = int(ds["n_rows"][k]), int(ds["n_p1"][k])
        t = ds["ms_rows"][k, :nr, None].astype(np.float64) + ds["ms_pass1"][k, None, :npp]
        if scores is None:
            ci = 0
        else:
            ci = int(np.argmin(scores[pos:pos + nr * npp]))
        pos += nr * npp
        out.append(t.ravel()[ci] / t.min() - 1.0)
    r = np.asarray(out)
    return {"mean": float(r.mean()), "median": float(np.median(r)), "p90": float(np.quantile(r, 0.9)),
            "max": float(r.max()), "zero_regret_frac": float((r <= 1e-9).mean()), "n": int(r.size)}


def standardise(X: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    mean = X.mean(axis=0)
    scale = X.std(axis=0)
    scale = np.where(scale > 1e-6, scale, 1.0)
    return mean.astype(np.float32), scale.astype(np.float32)


def train(ds: dict, train_idx, *, epochs: int = 300, batch: int = 1024, lr: float = 2e-3, seed: int = 0,
          log_every: int = 50) -> dict:
    import torch
    X, y, _ = compose(ds, train_idx)
    mean, scale = standardise(X)
    Xs = (X - mean) / scale
    dev = torch.device("cuda")
    Xd = torch.tensor(Xs, device=dev)
    yd = torch.tensor(y, device=dev)
    net = MLP(init_params(GBSP_N_FEATURES, seed))
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = Xd.shape[0]
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to(dev)
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / epochs))  # cosine decay
        tot = 0.0
        for b0 in range(0, n, batch):
            sel = perm[b0:b0 + batch]
            xb = Xd.index_select(0, sel).contiguous()
            tb = yd.index_select(0, sel).contiguous()
            net.backward(xb, tb)
            net.adam(lr_ep)
            tot += float(net.loss.item()) * xb.shape[0]
        hist.append(tot / n)
        if log_every and (ep + 1) % log_every == 0:
            print(f"train: epoch {ep + 1}/{epochs} mse(log ms) {hist[-1]:.5f}", flush=True)
    return {"params": net.params(), "mean": mean, "scale": scale, "loss_history": np.asarray(hist, np.float32),
            "lo": X.min(0), "hi": X.max(0)}


def predict(model: dict, X: np.ndarray) -> np.ndarray:
    """log ms predicted by the library's forward kernel."""
    import torch
    net = MLP(model["params"])
    Xs = torch.tensor((X - model["mean"]) / model["scale"], dtype=torch.float32, device="cuda")
    return net.forward(Xs).cpu().numpy()


# the library's rule (gbsp_cost_model_set_domain): a feature may leave the
# training range by at most this fraction of the range's width
DOMAIN_MARGIN = 0.1


def in_domain(model: dict, X: np.ndarray) -> bool:
    """True when every candidate's features lie in the model's training
    range (with the library's margin); always true without a range."""
    if "lo" not in model:
        return True
    m = DOMAIN_MARGIN * (model["hi"] - model["lo"])
    return bool(np.all((X >= model["lo"] - m) & (X <= model["hi"] + m)))


def save_model(path, model: dict, meta: dict) -> None:
    extra = {k: model[k] for k in ("lo", "hi") if k in model}
    np.savez(path, params=model["params"], mean=model["mean"], scale=model["scale"],
             loss_history=model.get("loss_history", np.zeros(0, np.float32)), meta=json.dumps(meta), **extra)


def load_model(path=DEFAULT_MODEL) -> dict:
    z = np.load(path, allow_pickle=False)
    m = {"params": z["params"].astype(np.float32), "mean": z["mean"].astype(np.float32),
         "scale": z["scale"].astype(np.float32), "meta": json.loads(str(z["meta"]))}
    if "lo" in z.files:  # training range of every feature (the planner's domain)
        m["lo"], m["hi"] = z["lo"].astype(np.float32), z["hi"].astype(np.float32)
    return m


def install(model: dict) -> None:
    """Makes `model` the one planner="learned" uses (process-wide)."""
    lib = load()
    fp = C.POINTER(C.c_float)
    p = np.ascontiguousarray(model["params"], np.float32)
    m = np.ascontiguousarray(model["mean"], np.float32)
    s = np.ascontiguousarray(model["scale"], np.float32)
    check(lib.gbsp_cost_model_set(p.ctypes.data_as(fp), GBSP_N_FEATURES, m.ctypes.data_as(fp),
                                  s.ctypes.data_as(fp)), "gbsp_cost_model_set")
    if "lo" in model:
        lo = np.ascontiguousarray(model["lo"], np.float32)
        hi = np.ascontiguousarray(model["hi"], np.float32)
        check(lib.gbsp_cost_model_set_domain(GBSP_N_FEATURES, lo.ctypes.data_as(fp), hi.ctypes.data_as(fp)),
              "gbsp_cost_model_set_domain")


_installed = False


def ensure_installed(path=DEFAULT_MODEL) -> None:
    global _installed
    if not _installed:
        if not Path(path).exists():
            raise RuntimeError(f"no trained cost model at {path}")
        install(load_model(path))
        _installed = True


def load_dataset(path=DEFAULT_DATA) -> dict:
    z = np.load(path, allow_pickle=False)
    return {k: z[k] for k in z.files}


def split(ds: dict) -> tuple[np.ndarray, np.ndarray]:
    n = len(ds["n_rows"])
    n_test = int(ds.get("n_test", np.int32(200)))
    return np.arange(0, n - n_test), np.arange(n - n_test, n)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(prog="python -m cuspfft_gb300.costmodel")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--out", required=True)
    c.add_argument("--train", type=int, default=2000)
    c.add_argument("--test", type=int, default=200)
    c.add_argument("--seed", type=int, default=7)
    c.add_argument("--reps", type=int, default=3)
    t = sub.add_parser("train")
    t.add_argument("--data", default=str(DEFAULT_DATA))
    t.add_argument("--out", default=str(DEFAULT_MODEL))
    t.add_argument("--epochs", type=int, default=300)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--large", action="store_true", help="also evaluate on the 40421 x 40421 matrix")
    a = ap.parse_args(argv)
    if a.cmd == "collect":
        mats = list(dataset_matrices(a.train + a.test, a.seed))
        ds = collect(mats, reps=a.reps)
        ds["n_test"] = np.int32(a.test)
        ds["seed"] = np.int32(a.seed)
        np.savez_compressed(a.out, **ds)
        print(f"wrote {a.out}")
    else:
        ds = load_dataset(a.data)
        tr, te = split(ds)
        model = train(ds, tr, epochs=a.epochs, seed=a.seed)
        Xt, _, _ = compose(ds, te)
        pred = predict(model, Xt)
        meta = {"train_matrices": int(tr.size), "test_matrices": int(te.size), "epochs": a.epochs,
                "regret_learned": regret(ds, te, pred), "regret_analytic": regret(ds, te)}
        if a.large:
            meta["large_matrix"] = evaluate_large(model)
        save_model(a.out, model, meta)
        print(json.dumps(meta))


def evaluate_large(model: dict) -> dict:
    """The 40421 x 40421 power-law adjacency (~351k nnz, 4-byte indices):
    exhaustive tuning against the learned planner's choice (the network's
    pick inside its training range, else the analytic one), the network's
    own pick and the analytic choice."""
    coo = synthetic.config_matrix("uniform_powerlaw_40421")
    ds = collect([coo], reps=2, log_every=0, index_bytes=4)
    X, _, _ = compose(ds, [0])
    pred = predict(model, X)
    nr, npp = int(ds["n_rows"][0]), int(ds["n_p1"][0])
    t = ds["ms_rows"][0, :nr, None].astype(np.float64) + ds["ms_pass1"][0, None, :npp]
    net_ms = float(t.ravel()[int(np.argmin(pred))])
    inside = in_domain(model, X)
    learned_ms = net_ms if inside else float(t[0, 0])
    return {"shape": [coo.rows, coo.cols], "nnz": coo.nnz, "index_bytes": 4, "candidates": nr * npp,
            "in_domain": inside, "best_ms": float(t.min()), "learned_ms": learned_ms,
            "network_ms": net_ms, "analytic_ms": float(t[0, 0]),
            "regret_learned": learned_ms / float(t.min()) - 1.0,
            "regret_network": net_ms / float(t.min()) - 1.0,
            "regret_analytic": float(t[0, 0] / t.min() - 1.0)}


if __name__ == "__main__":
    main()
