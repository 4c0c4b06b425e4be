"""Train the learned warm-start net on the c4 set and evaluate it with the
FIRE-finishes-and-judges protocol.

    python open-qmin_gb300/train_warmstart.py --train 4096 --test 256 --epochs 16 \\
        --out weights.npz --report report.json

Training data: c4 solves (64^3, homeotropic z-walls, one random homeotropic
sphere, random initial field) with seeds 0 .. train-1, minimised by the
batched FP32 FIRE path to forceMax < 1e-6; test solves use seeds
100000 .. 100000+test-1.  The weights file holds the FP32 parameter vector
(`params`), the layer table and the training history."""
import argparse
import importlib
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_package():
    if "qmin_gb300" in sys.modules:
        return sys.modules["qmin_gb300"]
    spec = importlib.util.spec_from_file_location("qmin_gb300", os.path.join(HERE, "__init__.py"),
                                                  submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["qmin_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--test", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=16)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--side", type=int, default=64)
    ap.add_argument("--no-augment", action="store_true")
    ap.add_argument("--out", required=True, help="weights file (.npz)")
    ap.add_argument("--report", default=None, help="JSON report of the evaluation")
    a = ap.parse_args(argv)
    q = load_package()
    import torch
    w = importlib.import_module("qmin_gb300.workloads")
    ws = importlib.import_module("qmin_gb300.warmstart")
    t0 = time.perf_counter()
    data = ws.make_dataset(lambda s: w.c4_solve(s, side=a.side), list(range(a.train)))
    t_data = time.perf_counter() - t0
    t1 = time.perf_counter()
    params, hist = ws.train(data, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, augment=not a.no_augment)
    t_train = time.perf_counter() - t1
    data_its = data["iterations"]
    del data
    torch.cuda.empty_cache()
    np.savez_compressed(a.out, params=params.astype(np.float32), layers=np.array(q.WARMNET_LAYERS, dtype=np.int32),
                        loss_history=np.array(hist), train=a.train, epochs=a.epochs, batch=a.batch, lr=a.lr,
                        side=a.side, seed=a.seed, augment=not a.no_augment)
    print(f"weights written to {a.out} (data {t_data:.0f} s, training {t_train:.0f} s)", flush=True)
    report = dict(train=a.train, test=a.test, epochs=a.epochs, data_seconds=t_data, train_seconds=t_train,
                  data_iterations_median=float(np.median(data_its)), loss_history=hist)
    if a.test > 0:
        test = [w.c4_solve(100000 + k, side=a.side) for k in range(a.test)]
        res = ws.evaluate(params, test)
        res["failed"] = [int(k) for k in res["failed"]]
        report["evaluation"] = res
    if a.report:
        with open(a.report, "w") as f:
            json.dump(report, f, indent=1, default=float)
    return report


if __name__ == "__main__":
    main()
