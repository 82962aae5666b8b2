"""CPU checks of the cost-model pieces: the FP64 MLP oracle against its own
finite differences, the structure features against a numpy restatement, the
tuner's configuration table, and the tuning database."""
import math
import os

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from matrixmultiplicationcuda_gb300 import costmodel, tuner
from oracle import mlp_oracle


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = mlp_oracle.dims_of(5, 7, 3, 4)
    n = 2 * 5 + 7 * 5 + 7 + 7 * 7 + 7 + 7 * 7 + 7 + 4 * 7 + 4
    p = rng.standard_normal(n) * 0.5
    p[:5] = rng.standard_normal(5)
    p[5:10] = rng.uniform(0.5, 2.0, 5)
    X = rng.standard_normal((9, 5))
    T = rng.standard_normal((9, 4))
    M = (rng.uniform(size=(9, 4)) > 0.3).astype(float)
    loss, g = mlp_oracle.loss_grad(dims, p, X, T, M)
    assert np.all(g[:10] == 0)
    h = 1e-6
    for k in rng.choice(np.arange(10, n), 40, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mlp_oracle.loss_grad(dims, pp, X, T, M)[0] - mlp_oracle.loss_grad(dims, pm, X, T, M)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def _features_np(rp, ci, M, K, bR, N):
    MB, KB = M // bR, K // 16
    cnt = np.diff(rp).astype(float)
    mean = cnt.mean()
    rows = np.repeat(np.arange(MB), np.diff(rp))
    band = np.abs(16.0 * ci - bR * rows).max() if len(ci) else 0.0
    runs = 0
    for r in range(MB):
        seg = ci[rp[r]:rp[r + 1]]
        if len(seg):
            runs += 1 + int(np.sum(np.diff(seg) != 1))
    nnzb = len(ci)
    return np.array([
        math.log2(M), math.log2(K), math.log2(N), bR == 16, bR == 32, bR == 64,
        math.log2(max(nnzb / (MB * KB), 2.0 ** -20)), math.log2(1 + mean),
        (cnt.std() / mean) if mean > 0 else 0.0, math.log2(1 + cnt.max()), band / K,
        float(np.mean(cnt == 0)), math.log2(nnzb / runs) if runs else 0.0,
        math.log2(MB * ((N + 255) // 256) / 152.0), (cnt.max() / mean) if mean > 0 else 0.0,
        len(np.unique(ci)) / KB, 2.0, 0.0], np.float64)


@pytest.mark.parametrize("M,bR,pattern,dens,param,N", [
    (1024, 16, m.PATTERN_RANDOM, 0.1, 0.0, 1024), (2048, 64, m.PATTERN_BAND, 0.05, 8.0, 256),
    (1024, 32, m.PATTERN_BLOCKDIAG, 0.0, 128.0, 512), (4096, 64, m.PATTERN_LOGNORMAL, 0.05, 1.5, 4096),
    (512, 16, m.PATTERN_RANDOM, 0.0, 0.0, 128)])
def test_features_match_numpy(M, bR, pattern, dens, param, N):
    rp, ci = m.gen_structure(M, M, bR, pattern, dens, param, seed=3)
    got = tuner.features_host(rp, ci, M, M, bR, N)
    ref = _features_np(rp, ci, M, M, bR, N)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
    e4 = tuner.features_host(rp, ci, M, M, bR, N, dtype=m.DType.E4M3)
    sp = tuner.features_host(rp, ci, M, M, bR, N, dtype=m.DType.F16_SPLIT)
    assert e4[16] == 1 and e4[17] == 0 and sp[16] == 2 and sp[17] == 1


def test_features_reject_bad_structure():
    rp = np.array([0, 2, 1], np.int32)
    with pytest.raises(ValueError):
        tuner.features_host(rp, np.array([0, 1], np.int32), 32, 64, 16, 64)
    with pytest.raises(ValueError):
        tuner.features_host(np.array([0, 0], np.int32), np.zeros(0, np.int32), 16, 64, 16, 64, dtype=9)
    with pytest.raises(ValueError):
        tuner.features_host(np.array([0, 1], np.int32), np.array([9], np.int32), 16, 64, 16, 64)


def test_config_table():
    cs = tuner.configs()
    assert len(cs) == 56
    assert sum(tuner.is_plan(c) for c in cs) == 7
    keys = {tuner.config_key(c) for c in cs}
    assert len(keys) == len(cs)
    for bR in (16, 32, 64):
        for dt in (m.DType.F16, m.DType.BF16, m.DType.E4M3, m.DType.F16_SPLIT):
            mask = tuner.supported_mask(bR, dt, 512)
            assert mask.any()
            assert mask[tuner.default_index(bR, dt, 512)]
    assert tuner.supported_mask(64, m.DType.F16, 512).sum() == 45
    assert tuner.supported_mask(64, m.DType.E4M3, 512).sum() == 35


def test_tune_db_roundtrip(tmp_path):
    path = os.path.join(str(tmp_path), "db.json")
    db = tuner.TuneDB(path)
    ms = np.array([1.0, np.inf, 0.5], np.float32)
    db.put("sig", ms, device="dev")
    db.save()
    db2 = tuner.TuneDB(path)
    np.testing.assert_array_equal(db2.get("sig", device="dev"), ms)
    assert db2.get("other", device="dev") is None


def test_regret_and_targets():
    T = np.array([[1.0, 2.0, np.inf], [3.0, 1.5, 1.0]], np.float32)
    Tl, mask = costmodel.targets(T)
    assert mask.tolist() == [[1, 1, 0], [1, 1, 1]]
    assert abs(Tl[0, 0] - math.log(1000.0)) < 1e-5
    r = costmodel.regret(T, np.array([1, 2]))
    np.testing.assert_allclose(r, [1.0, 0.0])


DATA = os.path.join(os.path.dirname(costmodel.__file__), "data")


def _committed():
    z = np.load(os.path.join(DATA, "tune_dataset.npz"))
    cm = np.load(os.path.join(DATA, "costmodel.npz"))
    from matrixmultiplicationcuda_gb300.costmodel_train import load_specs
    return z, cm, load_specs(z, "te_")


def test_committed_dataset_shape():
    z, cm, specs = _committed()
    assert z["F_train"].shape == (2000, tuner.N_FEATURES) and z["T_train"].shape == (2000, tuner.n_configs())
    assert z["F_test"].shape == (500, tuner.N_FEATURES) and z["T_test"].shape == (500, tuner.n_configs())
    assert list(cm["shape"]) == [tuner.N_FEATURES, 64, 3, tuner.n_configs()]
    # every product's measured entries are exactly the supported ones
    for i in range(0, 500, 25):
        sp = specs[i]
        mask = tuner.supported_mask(sp["bR"], sp["dtype"], sp["N"])
        assert np.array_equal(np.isfinite(z["T_test"][i]), mask)
    # features recomputed from the regenerated structure match the stored ones
    for i in range(0, 500, 50):
        sp = specs[i]
        rp, ci = m.gen_structure(sp["M"], sp["K"], sp["bR"], sp["pattern"], sp["density"], sp["param"],
                                 seed=sp["seed"])
        f = tuner.features_host(rp, ci, sp["M"], sp["K"], sp["bR"], sp["N"], sp["dtype"])
        np.testing.assert_array_equal(f, z["F_test"][i])


def test_committed_model_beats_heuristic_on_held_out():
    """The trained network (evaluated here by the FP64 oracle restatement)
    picks configurations on the 500 held-out products whose measured time is
    within 10 % of the exhaustive sweep's best on average, and better than the
    library's fixed heuristic."""
    z, cm, specs = _committed()
    s = cm["shape"]
    dims = mlp_oracle.dims_of(int(s[0]), int(s[1]), int(s[2]), int(s[3]))
    T = z["T_test"]
    pred = mlp_oracle.forward(dims, cm["params"].astype(np.float64), z["F_test"])
    _, mask = costmodel.targets(T)
    pick = costmodel.picks_from_predictions(pred, mask)
    heur = np.array([tuner.default_index(sp["bR"], sp["dtype"], sp["N"]) for sp in specs])
    r_model = costmodel.regret(T, pick)
    r_heur = costmodel.regret(T, heur)
    assert r_model.mean() <= 0.10
    assert np.mean(r_model <= 0.10) >= 0.85
    assert r_model.mean() < r_heur.mean() / 2
    assert np.exp(np.mean(np.log(T[np.arange(500), heur] / T[np.arange(500), pick]))) > 1.03
