"""Batched solve of a Hamiltonian family with a learned T2 guess.

Workflow for many related Hamiltonians of uneven size (B = B0 + s*B1 sliced to
no in [4, 12], nv in [20, 96], see generator.make_family):

1. every member is solved by the batched FP64 solver from the MP2 guess (one graph
   launch per sweep for all members);
2. the guess network is trained on the GPU on the converged amplitudes of the training
   members (pair features -> t2 - t2_mp2);
3. the test members are solved again, each from the network's guess, and compared with
   their MP2-guess solves: iterations, device time and energies (the plain iteration is
   the arbiter: both solves converge to the same R_CONVERGENCE).

    python -m ugacc_gb300.family --members 512 --train 384 --seed 7

prints one JSON object.  Rows of each training member are subsampled (--row-fraction)
to bound the host memory of the training set.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import ugacc_gb300 as U
from ugacc_gb300.generator import make_family


def run(members=512, train=384, seed=7, r_conv=1e-8, epochs=6, batch_rows=8192, lr=1e-3, row_fraction=0.25,
        no_range=(4, 12), nv_range=(20, 96), maxiter=100):
    fam = make_family(members, seed, no_range=no_range, nv_range=nv_range)
    opts = {"R_CONVERGENCE": r_conv, "MAXITER": maxiter}
    train_idx = list(range(train))
    test_idx = list(range(train, members))

    # 1. plain batched solve of every member from MP2
    t0 = time.time()
    bt = U.Batch()
    for h in fam:
        bt.add(h)
    load_s = time.time() - t0
    e_all, it_all, cv_all = bt.ccsd(opts)
    info_all = bt.info()

    # 2. training set from the converged training members
    rng = np.random.default_rng(seed)
    Xs, ts = [], []
    for k in train_idx:
        if not cv_all[k]:
            continue
        X, t = bt.features(k, with_targets=True)
        keep = rng.random(X.shape[0]) < row_fraction
        Xs.append(X[keep])
        ts.append(t[keep])
    X = np.concatenate(Xs)
    t = np.concatenate(ts)
    rows = int(X.shape[0])
    net = U.MLP(seed=seed)
    t1 = time.time()
    loss0, _ = net.loss_grad(X[:200000], t[:200000])
    loss = net.train(X, t, epochs=epochs, batch=batch_rows, lr=lr, seed=seed)
    train_s = time.time() - t1
    del X, t, Xs, ts
    bt.close()

    # 3. the test members: MP2 guess vs learned guess, each as one batch
    test = [fam[k] for k in test_idx]
    b_mp2 = U.Batch()
    for h in test:
        b_mp2.add(h)
    e_mp2, it_mp2, cv_mp2 = b_mp2.ccsd(opts)
    info_mp2 = b_mp2.info()
    b_mp2.close()
    b_mlp = U.Batch()
    for k, h in enumerate(test):
        b_mlp.add(h)
        b_mlp.guess(k, net)
    e_mlp, it_mlp, cv_mlp = b_mlp.ccsd(opts)
    info_mlp = b_mlp.info()
    b_mlp.close()

    return {
        "members": members, "train": train, "test": len(test_idx), "r_convergence": r_conv, "seed": seed,
        "all_members": {"converged": int(cv_all.sum()), "iterations_total": int(it_all.sum()),
                        "sweeps": info_all["sweeps"], "solve_s": info_all["solve_ms"] / 1e3,
                        "tflops": info_all["flops"] / (info_all["solve_ms"] / 1e3) / 1e12 if info_all["solve_ms"] else None,
                        "grouped_ops": info_all["grouped_ops"], "graph_kernels": info_all["graph_kernels"],
                        "shape_choice": info_all["shape_choice"], "load_s": load_s},
        "training": {"rows": rows, "loss_before": float(loss0),
                     "loss_after": float(loss), "epochs": epochs, "train_s": train_s},
        "test_mp2_guess": {"iterations_total": int(it_mp2.sum()), "iterations_mean": float(it_mp2.mean()),
                           "sweeps": info_mp2["sweeps"], "solve_s": info_mp2["solve_ms"] / 1e3,
                           "converged": int(cv_mp2.sum())},
        "test_learned_guess": {"iterations_total": int(it_mlp.sum()), "iterations_mean": float(it_mlp.mean()),
                               "sweeps": info_mlp["sweeps"], "solve_s": info_mlp["solve_ms"] / 1e3,
                               "converged": int(cv_mlp.sum())},
        "iterations_saved": int(it_mp2.sum() - it_mlp.sum()),
        "max_abs_dE": float(np.max(np.abs(e_mlp - e_mp2))),
    }


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--train", type=int, default=384)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--r-conv", type=float, default=1e-8)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--row-fraction", type=float, default=0.25)
    ap.add_argument("--no-max", type=int, default=12)
    ap.add_argument("--nv-max", type=int, default=96)
    a = ap.parse_args(argv)
    out = run(a.members, a.train, a.seed, a.r_conv, a.epochs, row_fraction=a.row_fraction,
              no_range=(4, a.no_max), nv_range=(20, a.nv_max))
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
