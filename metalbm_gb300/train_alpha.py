"""Train the committed alpha-guess model from a plain entropic run.

The training data follow the entropic workload: D3Q27 entropic SRT,
beta = 0.9995, Taylor-Green vortex U0 = 0.05 on [0, 2pi)^3 (with
--perturbation, plus the random-phase solenoidal perturbation of amplitude
1e-3 on the shell 8 <= |k| <= 10, seed 2, of the learned-alpha benchmark),
every node solving for alpha in FP64 to |F| <= 1e-12 with the bisection
fallback; every
`--every` steps, `--samples` uniformly drawn nodes are logged as
(f_neq/rho, alpha*) pairs. The network is trained on the GPU with the
library's own kernels and saved to metalbm_gb300/models/alpha_d3q27.npz.

Usage: python -m metalbm_gb300.train_alpha [--size 256] [--steps 2000]
           [--every 200] [--samples 1000000] [--storage f64] [--perturbation]
           [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import alpha_model, fields
from .lattice import InputDeck


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=200)
    ap.add_argument("--samples", type=int, default=1000000)
    ap.add_argument("--storage", default="f64")
    ap.add_argument("--perturbation", action="store_true",
                    help="add the benchmark's solenoidal perturbation (1e-3 on 8 <= |k| <= 10)")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default=str(alpha_model.default_model_path("D3Q27")))
    args = ap.parse_args()
    shape = (args.size,) * 3
    deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=1.0 / (2 * 0.9995),
                     globalLength=shape, storage=args.storage, alphaSolver="residual",
                     alphaGuess="previous", newtonTolerance=1e-12, deviationThreshold=0.0)
    rho, u = fields.taylor_green(shape, u0=0.05)
    if args.perturbation:
        u = u + fields.solenoidal_shell(shape, 8.0, 10.0, 1e-3, seed=2)
    t0 = time.time()
    X, y = alpha_model.collect_samples(deck, rho, u, steps=args.steps, every=args.every,
                                       n_per_log=args.samples)
    t1 = time.time()
    model, loss = alpha_model.fit(X, y, deck, epochs=args.epochs)
    t2 = time.time()
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    alpha_model.save_model(model, out, samples=len(y), grid=args.size, steps=args.steps,
                           every=args.every, storage=args.storage, final_loss=loss,
                           perturbation=int(args.perturbation))
    print(json.dumps({"samples": int(len(y)), "alpha_min": float(y.min()),
                      "alpha_max": float(y.max()), "alpha_std": float(y.std()),
                      "final_mse": float(loss), "rmse_over_std": float(np.sqrt(loss) / max(y.std(), 1e-30)),
                      "collect_s": t1 - t0, "train_s": t2 - t1, "out": str(out)}))


if __name__ == "__main__":
    main()
