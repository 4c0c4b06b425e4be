"""Train the learned warm-start net on the c4 set and evaluate it with the
FIRE-finishes-and-judges protocol.

    python open-qmin_gb300/train_warmstart.py --train 4096 --test 256 --epochs 16 \\
        --out weights.npz --report report.json

Training data: c4 solves (64^3, homeotropic z-walls, one random homeotropic
sphere, random initial field) with seeds 0 .. train-1, minimised by the
batched FP32 FIRE path to forceMax < 1e-6; test solves use seeds
100000 .. 100000+test-1.  The weights file holds the FP32 parameter vector
(`params`), the layer table and the training history.

Patch-tiled fine-tuning on the large configurations:

    python open-qmin_gb300/train_warmstart.py --finetune-from weights/warmnet_c4.npz \
        --train 256 --crops-c2 12 --crops-c5 2 --epochs 6 --lr 3e-4 --out tuned.npz

adds 64^3 crops of whole 200^3 c2 lattices (seeds 1..n, each minimised whole
by FP32 FIRE) and of 400^3 c5 lattices (seeds 1..n; 8 spheres, E field) to
the c4 samples, with an 8-site band at every crop face left out of the loss,
and starts from the given weights."""
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
    ap.add_argument("--finetune-from", default=None, help="weights file (.npz) to start from")
    ap.add_argument("--crops-c2", type=int, default=0, help="200^3 c2 lattices (seeds 1..n) cut into 64^3 crops")
    ap.add_argument("--crops-c5", type=int, default=0, help="400^3 c5 lattices (seeds 1..n) cut into 64^3 crops")
    ap.add_argument("--out", required=True, help="weights file (.npz)")
    ap.add_argument("--report", default=None, help="JSON report of the evaluation")
    a = ap.parse_args(argv)
    q = load_package()
    import torch
    w = importlib.import_module("qmin_gb300.workloads")
    ws = importlib.import_module("qmin_gb300.warmstart")
    t0 = time.perf_counter()
    parts = []
    if a.train > 0:
        parts.append(ws.make_dataset(lambda s: w.c4_solve(s, side=a.side), list(range(a.train))))
    if a.crops_c2 > 0:
        parts.append(ws.make_crop_dataset([w.c2_lattice(200, seed=s) for s in range(1, a.crops_c2 + 1)],
                                          side=a.side))
    if a.crops_c5 > 0:
        parts.append(ws.make_crop_dataset([w.c5_lattice(400, seed=s) for s in range(1, a.crops_c5 + 1)],
                                          side=a.side))
    data = parts[0] if len(parts) == 1 else ws.concat_datasets(parts)
    t_data = time.perf_counter() - t0
    p0 = None if a.finetune_from is None else np.load(a.finetune_from)["params"]
    t1 = time.perf_counter()
    params, hist = ws.train(data, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, params=p0,
                            augment=not a.no_augment)
    t_train = time.perf_counter() - t1
    data_its = data["iterations"]
    del data
    torch.cuda.empty_cache()
    np.savez_compressed(a.out, params=params.astype(np.float32), layers=np.array(q.WARMNET_LAYERS, dtype=np.int32),
                        loss_history=np.array(hist), train=a.train, epochs=a.epochs, batch=a.batch, lr=a.lr,
                        side=a.side, seed=a.seed, augment=not a.no_augment, crops_c2=a.crops_c2,
                        crops_c5=a.crops_c5, finetune_from=str(a.finetune_from))
    print(f"weights written to {a.out} (data {t_data:.0f} s, training {t_train:.0f} s)", flush=True)
    report = dict(train=a.train, test=a.test, epochs=a.epochs, data_seconds=t_data, train_seconds=t_train,
                  crops_c2=a.crops_c2, crops_c5=a.crops_c5, samples=int(len(data_its)) if a.train else None,
                  data_iterations_median=float(np.median(data_its)) if len(data_its) else None,
                  loss_history=hist)
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
