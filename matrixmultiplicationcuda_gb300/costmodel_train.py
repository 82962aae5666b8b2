"""Collects the cost model's training data, trains it and measures its regret.

    python -m matrixmultiplicationcuda_gb300.costmodel_train [--out DIR]
        [--n-train 2000] [--n-test 500] [--seed 11] [--steps 8000]
        [--mode b2b|cold] [--dataset PATH]   # reuse collected sweeps instead of collecting

1. Draws n_train + n_test seeded synthetic products (costmodel.sample_specs)
   and sweeps every tuner configuration on each (the autotuner's own timings),
   by default back to back over rotating copies with plans chained by the
   inputs-ready flag (the regime of the benchmark's timed loop).
2. Trains the MLP on the first n_train with the library's CUDA kernels.
3. On the n_test held-out products compares three ways of choosing a
   configuration against the exhaustive sweep's best: the trained model, the
   library's fixed heuristic (spmm_default_config) and, as a floor, the best
   single configuration of the training set. Regret = t(choice) / t(best) - 1.
Writes DIR/tune_dataset.npz, DIR/costmodel.npz and DIR/costmodel_report.json.
"""
import argparse
import json
import os
import time

import numpy as np

from . import costmodel, tuner

HERE = os.path.dirname(os.path.abspath(__file__))


def spec_arrays(specs):
    keys = ["M", "K", "N", "bR", "pattern", "density", "param", "seed", "dtype"]
    return {"spec_" + k: np.array([s[k] for s in specs]) for k in keys}


def load_specs(z, prefix):
    keys = [k for k in z.files if k.startswith(prefix + "spec_")]
    n = len(z[keys[0]])
    return [{k[len(prefix) + 5:]: z[k][i].item() for k in keys} for i in range(n)]


def regret_stats(r):
    return {"mean": float(np.mean(r)), "median": float(np.median(r)), "p90": float(np.quantile(r, 0.9)),
            "max": float(np.max(r)), "within_10pct": float(np.mean(r <= 0.10))}


def evaluate(F, T, nnzb, specs, params, s, device="cuda"):
    """Regret of the model, the heuristic and the best fixed config on (F, T)."""
    import torch
    net = costmodel.MLP(s, params, device=device)
    pred = net.forward(torch.from_numpy(F).to(device)).cpu().numpy()
    _, mask = costmodel.targets(T)
    pick = costmodel.picks_from_predictions(pred, mask)
    heur = np.array([tuner.default_index(sp["bR"], sp["dtype"], sp["N"]) for sp in specs])
    r_model = costmodel.regret(T, pick)
    r_heur = costmodel.regret(T, heur)
    flops = np.array([2.0 * n * sp["bR"] * 16 * sp["N"] for n, sp in zip(nnzb, specs)])
    t_model = T[np.arange(len(pick)), pick]
    t_heur = T[np.arange(len(heur)), heur]
    t_best = np.min(T, axis=1)
    return {
        "model_regret": regret_stats(r_model),
        "heuristic_regret": regret_stats(r_heur),
        "geomean_speedup_model_over_heuristic": float(np.exp(np.mean(np.log(t_heur / t_model)))),
        "total_time_ms": {"model": float(t_model.sum()), "heuristic": float(t_heur.sum()),
                          "sweep_best": float(t_best.sum())},
        "aggregate_tflops": {"model": float(flops.sum() / t_model.sum() / 1e9),
                             "heuristic": float(flops.sum() / t_heur.sum() / 1e9),
                             "sweep_best": float(flops.sum() / t_best.sum() / 1e9)},
    }, pick, heur


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "data"))
    ap.add_argument("--n-train", type=int, default=2000)
    ap.add_argument("--n-test", type=int, default=500)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--dataset", default=None)
    ap.add_argument("--mode", default="b2b", choices=["b2b", "cold"])
    args = ap.parse_args(argv)
    import torch
    os.makedirs(args.out, exist_ok=True)
    dev = "cuda"
    t0 = time.time()
    if args.dataset:
        z = np.load(args.dataset)
        Ftr, Ttr, ntr = z["F_train"], z["T_train"], z["nnzb_train"]
        Fte, Tte, nte = z["F_test"], z["T_test"], z["nnzb_test"]
        str_, ste = load_specs(z, "tr_"), load_specs(z, "te_")
    else:
        str_ = costmodel.sample_specs(args.n_train, args.seed)
        ste = costmodel.sample_specs(args.n_test, args.seed + 1)
        Ftr, Ttr, ntr = costmodel.collect(str_, progress=250, mode=args.mode)
        Fte, Tte, nte = costmodel.collect(ste, progress=250, mode=args.mode)
        arrays = {}
        for pfx, sp in (("tr_", str_), ("te_", ste)):
            for k, v in spec_arrays(sp).items():
                arrays[pfx + k] = v
        np.savez_compressed(os.path.join(args.out, "tune_dataset.npz"), F_train=Ftr, T_train=Ttr,
                            nnzb_train=ntr, F_test=Fte, T_test=Tte, nnzb_test=nte,
                            device=np.array(torch.cuda.get_device_name()), regime=np.array(args.mode),
                            **arrays)
    t_collect = time.time() - t0

    s = costmodel.shape()
    mu = Ftr.mean(axis=0)
    sigma = Ftr.std(axis=0)
    sigma = np.where(sigma > 1e-3, sigma, 1.0).astype(np.float32)
    p0 = costmodel.init_params(s, mu, sigma, seed=args.seed)
    net = costmodel.MLP(s, p0, device=dev)
    Tl, M = costmodel.targets(Ttr)
    Xt, Tt, Mt = (torch.from_numpy(a).to(dev) for a in (Ftr, Tl, M))
    t1 = time.time()
    losses = net.train(Xt, Tt, Mt, steps=args.steps, batch=256, lr=2e-3, wd=1e-4, seed=args.seed,
                       log_every=max(1, args.steps // 20))
    torch.cuda.synchronize()
    t_train = time.time() - t1
    params = net.host_params()
    costmodel.save(os.path.join(args.out, "costmodel.npz"), s, params)

    rep_test, pick, heur = evaluate(Fte, Tte, nte, ste, params, s, dev)
    rep_train, _, _ = evaluate(Ftr, Ttr, ntr, str_, params, s, dev)
    # the best single configuration on the training set, applied to the held-out set
    _, Mtr = costmodel.targets(Ttr)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = Ttr / np.min(Ttr, axis=1, keepdims=True)
    fixed_scores = np.where(Mtr > 0, np.log(rel), 10.0).mean(axis=0)
    fixed = int(np.argmin(fixed_scores))
    _, Mte = costmodel.targets(Tte)
    fixed_pick = np.where(Mte[:, fixed] > 0, fixed, heur)
    report = {
        "device": torch.cuda.get_device_name(),
        "regime": (str(z["regime"]) if args.dataset and "regime" in z.files else args.mode),
        "n_train": len(Ftr), "n_test": len(Fte), "configs": tuner.n_configs(),
        "features": tuner.N_FEATURES, "hidden": s.hidden, "layers": s.layers, "steps": args.steps,
        "collect_s": t_collect, "train_s": t_train,
        "train_loss": losses,
        "test": rep_test,
        "train": rep_train,
        "best_fixed_config": {"index": fixed, "name": tuner.config_name(tuner.configs()[fixed]),
                              "test_regret": regret_stats(costmodel.regret(Tte, fixed_pick))},
    }
    with open(os.path.join(args.out, "costmodel_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps({k: report[k] for k in ("n_train", "n_test", "collect_s", "train_s")}))
    print("test  model regret", json.dumps(rep_test["model_regret"]))
    print("test  heuristic   ", json.dumps(rep_test["heuristic_regret"]))
    print("test  fixed best  ", json.dumps(report["best_fixed_config"]))
    print("test  speedup model/heuristic %.3f" % rep_test["geomean_speedup_model_over_heuristic"])
    print("train model regret", json.dumps(rep_train["model_regret"]))


if __name__ == "__main__":
    main()
