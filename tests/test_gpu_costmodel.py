"""The cost model's CUDA kernels against the FP64 oracle (forward, loss,
gradient, AdamW), the device features, the sweep, and model-driven config
selection."""
import ctypes
import math

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from matrixmultiplicationcuda_gb300 import costmodel, tuner
from oracle import mlp_oracle, oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _random_model(seed, n_in=18, hidden=64, layers=3, n_out=None, batch=300):
    n_out = tuner.n_configs() if n_out is None else n_out
    rng = np.random.default_rng(seed)
    s = costmodel.shape(n_out=n_out, n_in=n_in, hidden=hidden, layers=layers)
    mu = rng.standard_normal(n_in).astype(np.float32)
    sigma = rng.uniform(0.5, 2.0, n_in).astype(np.float32)
    p = costmodel.init_params(s, mu, sigma, seed=seed)
    p[2 * n_in:] += (rng.standard_normal(p.size - 2 * n_in) * 0.05).astype(np.float32)
    X = (rng.standard_normal((batch, n_in)) * 2).astype(np.float32)
    T = rng.standard_normal((batch, n_out)).astype(np.float32)
    M = (rng.uniform(size=(batch, n_out)) > 0.25).astype(np.float32)
    return s, p, X, T, M, mlp_oracle.dims_of(n_in, hidden, layers, n_out)


@pytest.mark.parametrize("batch", [1, 63, 300, 2000])
def test_mlp_forward_matches_oracle(dev, batch):
    s, p, X, _, _, dims = _random_model(1, batch=batch)
    net = costmodel.MLP(s, p, device=dev)
    Y = net.forward(torch.from_numpy(X).to(dev)).cpu().numpy()
    ref = mlp_oracle.forward(dims, p, X)
    assert np.abs(Y - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("dims", [(18, 64, 3, 41), (5, 7, 2, 3), (16, 128, 1, 40)])
def test_mlp_gradient_matches_oracle(dev, dims):
    """The gradient check: loss and every parameter's gradient from the CUDA
    backward pass against the FP64 oracle's analytic gradient (itself checked
    against finite differences on the CPU)."""
    s, p, X, T, M, odims = _random_model(2, *dims, batch=500)
    net = costmodel.MLP(s, p, device=dev)
    loss, g = net.loss_grad(torch.from_numpy(X).to(dev), torch.from_numpy(T).to(dev), torch.from_numpy(M).to(dev))
    rl, rg = mlp_oracle.loss_grad(odims, p.astype(np.float64), X, T, M)
    assert abs(float(loss) - rl) <= 1e-5 * max(1.0, abs(rl))
    g = g.cpu().numpy()
    assert np.all(g[:2 * dims[0]] == 0)
    err = np.abs(g - rg).max() / np.abs(rg).max()
    assert err <= 1e-4, err


def test_mlp_gradient_deterministic(dev):
    s, p, X, T, M, _ = _random_model(3, batch=700)
    net = costmodel.MLP(s, p, device=dev)
    args = [torch.from_numpy(a).to(dev) for a in (X, T, M)]
    _, g1 = net.loss_grad(*args)
    _, g2 = net.loss_grad(*args)
    assert torch.equal(g1, g2)


def test_adam_step_matches_formula(dev):
    rng = np.random.default_rng(4)
    n, off = 1000, 32
    p = rng.standard_normal(n).astype(np.float32)
    g = rng.standard_normal(n).astype(np.float32)
    m0 = (rng.standard_normal(n) * 0.1).astype(np.float32)
    v0 = rng.uniform(0, 0.1, n).astype(np.float32)
    tp, tg, tm, tv = (torch.from_numpy(a.copy()).to(dev) for a in (p, g, m0, v0))
    lr, b1, b2, eps, wd, step = 1e-2, 0.9, 0.999, 1e-8, 1e-3, 7
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    m.check(m.lib().spmm_mlp_adam(vp(tp), vp(tg), vp(tm), vp(tv), n, off, lr, b1, b2, eps, wd, step, None))
    torch.cuda.synchronize()
    mm = b1 * m0 + (1 - b1) * g
    vv = b2 * v0 + (1 - b2) * g * g
    ref = p - lr * ((mm / (1 - b1 ** step)) / (np.sqrt(vv / (1 - b2 ** step)) + eps) + wd * p)
    out = tp.cpu().numpy()
    np.testing.assert_array_equal(out[:off], p[:off])
    np.testing.assert_allclose(out[off:], ref[off:], rtol=1e-5, atol=1e-6)


def test_mlp_training_fits_a_teacher(dev):
    """Training with the library's kernels drives the loss on a teacher
    network's outputs down by more than an order of magnitude."""
    s, pt, X, _, _, dims = _random_model(5, batch=2000)
    T = mlp_oracle.forward(dims, pt, X).astype(np.float32)
    M = np.ones_like(T)
    p0 = costmodel.init_params(s, pt[:18], pt[18:36], seed=9)
    net = costmodel.MLP(s, p0, device=dev)
    Xt, Tt, Mt = (torch.from_numpy(a).to(dev) for a in (X, T, M))
    l0 = float(net.loss_grad(Xt, Tt, Mt)[0])
    net.train(Xt, Tt, Mt, steps=1500, batch=256, lr=3e-3, wd=0.0, seed=1)
    l1 = float(net.loss_grad(Xt, Tt, Mt)[0])
    assert l1 < l0 / 20, (l0, l1)


def _product(dev, M, K, bR, pattern, dens, param, N, seed):
    rp, ci = m.gen_structure(M, K, bR, pattern, dens, param, seed=seed)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=seed + 1)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=seed + 2)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16, device=dev)
    B = torch.from_numpy(Bf).to(dev).half()
    return A, B, rp, ci, vals, Bf


def test_device_features_match_host(dev):
    A, B, rp, ci, _, _ = _product(dev, 2048, 2048, 32, m.PATTERN_LOGNORMAL, 0.05, 1.5, 512, 11)
    np.testing.assert_array_equal(tuner.features(A, 512), tuner.features_host(rp, ci, 2048, 2048, 32, 512))


@pytest.mark.parametrize("bR", [16, 64])
def test_sweep_times_supported_configs(dev, bR):
    A, B, rp, ci, vals, Bf = _product(dev, 1024, 2048, bR, m.PATTERN_RANDOM, 0.05, 0.0, 256, 13)
    C = torch.empty((1024, 256), dtype=torch.float32, device=dev)
    ms = tuner.sweep(A, B, 256, C, warmup=1, reps=3)
    mask = tuner.supported_mask(bR, m.DType.F16, 256)
    assert np.all(np.isfinite(ms[mask])) and np.all(ms[mask] > 0)
    assert np.all(np.isinf(ms[~mask]))
    # the last configuration swept left a correct product in C
    ref = oracle.bcsr_matmul_f64(rp, ci, torch.from_numpy(vals).half().double().numpy(), bR, 16,
                                 torch.from_numpy(Bf).half().double().numpy())
    mx, fr = oracle.rel_errors(C.cpu().numpy(), ref)
    assert mx <= 1e-5 and fr <= 1e-5


@pytest.mark.parametrize("bR,dtype", [(64, m.DType.F16), (16, m.DType.F16), (64, m.DType.E4M3)])
def test_back_to_back_sweep(dev, bR, dtype):
    """spmm_tune_sweep_b2b: every supported entry (plans included) timed over
    rotating copies, +inf elsewhere, and every copy's C left correct."""
    M, K, N = 1024, 2048, 256
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_RANDOM, 0.05, 0, seed=13)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=14)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=15)
    copies = []
    for _ in range(3):
        A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)
        Bq, _, Bs = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), dtype)
        copies.append((A, Bq.view(K, N), torch.full((M, N), float("nan"), device=dev), None,
                       float(Bs[0]) if Bs is not None else 1.0))
    ms = tuner.sweep_b2b(copies, launches=6, warmup=1)
    m.device_error_check()
    mask = tuner.supported_mask(bR, dtype, N)
    assert np.all(np.isfinite(ms[mask])) and np.all(ms[mask] > 0)
    assert np.all(np.isinf(ms[~mask]))
    assert any(tuner.is_plan(c) for c, ok in zip(tuner.configs(), mask) if ok)
    A0 = copies[0][0]
    if dtype == m.DType.E4M3:
        sv = A0.vals.view(torch.float8_e4m3fn).double().cpu().numpy().reshape(-1, bR * 16)
        sv = (sv * A0.scales.double().cpu().numpy()[:, None]).reshape(-1)
        sB = copies[0][1].view(torch.float8_e4m3fn).double().cpu().numpy() * copies[0][4]
    else:
        sv = A0.vals.double().cpu().numpy()
        sB = copies[0][1].double().cpu().numpy()
    ref = oracle.bcsr_matmul_f64(rp, ci, sv, bR, 16, sB)
    for A, B, C, _, _ in copies:
        mx, fr = oracle.rel_errors(C.cpu().numpy(), ref)
        assert mx <= 1e-5 and fr <= 1e-5


def test_cost_model_select_returns_supported_config(dev):
    s, p, _, _, _, _ = _random_model(7)
    cm = costmodel.CostModel(s, p)
    for bR in (16, 32, 64):
        A, B, *_ = _product(dev, 1024, 1024, bR, m.PATTERN_RANDOM, 0.1, 0.0, 512, 17)
        c, pred = cm.select(A, 512, return_predictions=True)
        mask = tuner.supported_mask(bR, m.DType.F16, 512)
        assert np.all(np.isinf(pred[~mask])) and np.all(np.isfinite(pred[mask]))
        i = int(np.argmin(pred))
        assert tuner.config_key(c) == tuner.config_key(tuner.configs()[i])
        C = m.spmm(A, B, cfg=c)
        m.device_error_check()
        assert torch.isfinite(C).all()
    cm.close()


def test_training_on_sweeps_gains_over_heuristic(dev):
    """Retrains the network from the committed sweep timings with the
    library's kernels: on the held-out products its picks beat the fixed
    heuristic's and stay within 10 % of the sweep's best on average."""
    import os
    from matrixmultiplicationcuda_gb300.costmodel_train import load_specs
    z = np.load(os.path.join(os.path.dirname(costmodel.__file__), "data", "tune_dataset.npz"))
    F, T = z["F_train"], z["T_train"]
    s = costmodel.shape()
    sigma = F.std(axis=0)
    p0 = costmodel.init_params(s, F.mean(axis=0), np.where(sigma > 1e-3, sigma, 1.0), seed=3)
    net = costmodel.MLP(s, p0, device=dev)
    Tl, M = costmodel.targets(T)
    net.train(*(torch.from_numpy(a).to(dev) for a in (F, Tl, M)), steps=3000, batch=256, lr=2e-3, seed=3)
    Tt = z["T_test"]
    pred = net.forward(torch.from_numpy(z["F_test"]).to(dev)).cpu().numpy()
    _, mt = costmodel.targets(Tt)
    pick = costmodel.picks_from_predictions(pred, mt)
    specs = load_specs(z, "te_")
    heur = np.array([tuner.default_index(sp["bR"], sp["dtype"], sp["N"]) for sp in specs])
    r_model, r_heur = costmodel.regret(Tt, pick), costmodel.regret(Tt, heur)
    assert r_model.mean() <= 0.10 and r_model.mean() < r_heur.mean() / 2, (r_model.mean(), r_heur.mean())


def test_committed_model_in_library_matches_oracle_pick(dev):
    """spmm_cost_model_select (features + the network on the GPU) picks the
    configuration the FP64 oracle network picks for the same features."""
    import os
    path = os.path.join(os.path.dirname(costmodel.__file__), "data", "costmodel.npz")
    cm = costmodel.CostModel.load(path)
    z = np.load(path)
    dims = mlp_oracle.dims_of(*[int(v) for v in z["shape"]])
    for (M, bR, pat, dens, param, N) in [(4096, 64, m.PATTERN_RANDOM, 0.02, 0.0, 512),
                                         (2048, 16, m.PATTERN_BAND, 0.05, 8.0, 1024),
                                         (8192, 32, m.PATTERN_LOGNORMAL, 0.05, 1.5, 256)]:
        A, B, rp, ci, _, _ = _product(dev, M, M, bR, pat, dens, param, N, 23)
        c, pred = cm.select(A, N, return_predictions=True)
        f = tuner.features_host(rp, ci, M, M, bR, N)
        ref = mlp_oracle.forward(dims, z["params"].astype(np.float64), f[None])[0]
        mask = tuner.supported_mask(bR, m.DType.F16, N)
        np.testing.assert_allclose(np.log(pred[mask] * 1e3), ref[mask], rtol=0, atol=1e-4)
        i = int(np.argmin(np.where(mask, ref, np.inf)))
        assert tuner.config_key(c) == tuner.config_key(tuner.configs()[i])
    cm.close()
