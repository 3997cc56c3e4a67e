"""Learned alpha guess: training data from a plain entropic run, GPU training,
and the committed model file.

The model maps a node's non-equilibrium deviations normalised by density,
x_q = f_neq_q / rho, to a starting guess for the entropic alpha root-find
(Collision.h:351-375). Training pairs (x, alpha*) are logged by a plain
entropic run (the sample logger of mlbm_step, MLBM_STEP_LOG_SAMPLES) and the
network is trained on the GPU by the library's own forward / backward / Adam
kernels (mlbm_train_alpha_model).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .lattice import InputDeck, Lattice, MlpModel

MODEL_DIR = Path(__file__).resolve().parent / "models"


def save_model(model: MlpModel, path: Path, **meta):
    np.savez(path, n_in=model.n_in, input_scale=model.input_scale, w1=model.w1, b1=model.b1,
             w2=model.w2, b2=model.b2, w3=model.w3, b3=np.float32(model.b3),
             output_scale=np.float32(model.output_scale),
             **{f"meta_{k}": np.asarray(v) for k, v in meta.items()})


def load_model(path: Path) -> MlpModel:
    z = np.load(path)
    return MlpModel(int(z["n_in"]), z["input_scale"], z["w1"], z["b1"], z["w2"], z["b2"],
                    z["w3"], float(z["b3"]), float(z["output_scale"]))


def default_model_path(lattice: str = "D3Q27") -> Path:
    return MODEL_DIR / f"alpha_{lattice.lower()}.npz"


def collect_samples(deck: InputDeck, rho: np.ndarray, u: np.ndarray, steps: int, every: int,
                    n_per_log: int, seed: int = 0):
    """Run the plain entropic method and log (f_neq/rho, alpha*) at n_per_log
    uniformly drawn nodes every `every` steps. Returns X [n, Q], y [n] of the
    nodes that went through the alpha solve."""
    rng = np.random.default_rng(seed)
    Xs, ys = [], []
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        done = 0
        while done < steps:
            n = min(every, steps - done)
            nodes = rng.choice(lat.V, size=min(n_per_log, lat.V), replace=False)
            lat.set_sample_nodes(np.sort(nodes))
            lat.step(n, samples=True)
            feat, alpha, solved = lat.samples()
            keep = solved.astype(bool)
            Xs.append(feat[keep])
            ys.append(alpha[keep])
            done += n
    return np.concatenate(Xs), np.concatenate(ys)


def fit(X: np.ndarray, y: np.ndarray, deck: InputDeck, epochs: int = 30, batch: int = 8192,
        lr: float = 2e-3, seed: int = 0) -> tuple[MlpModel, float]:
    """Train on the GPU. Inputs are scaled by 1/std per population; the output
    is 2 + output_scale * net(x) with output_scale = std(alpha* - 2)."""
    std = X.std(axis=0)
    input_scale = np.where(std > 0, 1.0 / np.maximum(std, 1e-30), 0.0).astype(np.float32)
    out_scale = float(max(np.std(y - 2.0), 1e-6))
    model = MlpModel.init(X.shape[1], input_scale, out_scale, seed=seed)
    small = InputDeck(latticeT=deck.latticeT, globalLength=(4, 4, 4), device=deck.device)
    with Lattice(small) as lat:
        model, loss = lat.train_alpha_model(X.astype(np.float32), y.astype(np.float32), model,
                                            epochs=epochs, batch=batch, lr=lr, seed=seed)
    return model, loss
