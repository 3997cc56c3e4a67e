"""Error of the reduced-precision storage formats against the FP64 step.

Two studies, each run on one GPU from the same seeded initial fields:

* ``bgk``: D3Q19 SRT-BGK with Guo forcing and the Kolmogorov force
  F_x(z) = 1e-6 sin(2 pi 2 z / L) (wavelength L/2, along z), tau = 0.55,
  rho = 1 and u uniform in [-1e-4, 1e-4] per component (seed 1), f at
  equilibrium. FP32 and FP16-shifted storage against FP64 storage at the
  given steps: the relative L2 error of u, the relative error of the total
  energy (1/V) sum 1/2 rho |u|^2, and the relative L2 error of the
  shell-averaged energy spectrum (the analysis of Analysis.h:122-177).
* ``entropic``: D3Q27 entropic SRT with beta = 0.9995, the Taylor-Green
  vortex (U0 = 0.05) plus a random-phase solenoidal perturbation of amplitude
  1e-3 on shells 8 <= |k| <= 10 (seed 2); FP32 storage with the learned alpha
  guess against FP64 storage (both with the residual solver, tolerance 1e-12):
  the same errors.

Usage: python -m metalbm_gb300.precision_study bgk --grid 256 --steps 500 1000 2000
       python -m metalbm_gb300.precision_study entropic --grid 256 --steps 50 100 200
Prints one JSON line per (storage, step).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import alpha_model, fields, spectral
from .lattice import InputDeck, Lattice


def _errors(ref: dict, got: dict, shape, torch=None) -> dict:
    u_r, u_g = ref["u"], got["u"]
    l2_u = float(np.linalg.norm(u_g - u_r) / np.linalg.norm(u_r))
    max_u = float(np.abs(u_g - u_r).max())
    e_r = spectral.energy(ref["rho"], u_r)
    e_g = spectral.energy(got["rho"], u_g)
    if torch is not None and torch.cuda.is_available():
        dev = torch.device("cuda")
        s_r = spectral.energy_spectrum(torch.from_numpy(u_r).to(dev), shape)
        s_g = spectral.energy_spectrum(torch.from_numpy(u_g).to(dev), shape)
    else:
        s_r = spectral.energy_spectrum(u_r, shape)
        s_g = spectral.energy_spectrum(u_g, shape)
    spec = float(np.linalg.norm(s_g - s_r) / np.linalg.norm(s_r))
    return {"u_l2_rel": l2_u, "u_max_abs": max_u, "u_max": float(np.abs(u_r).max()),
            "energy_rel": abs(e_g - e_r) / abs(e_r), "spectrum_l2_rel": spec,
            "energy": e_g, "energy_f64": e_r}


def bgk_decks(n: int):
    common = dict(latticeT="D3Q19", collisionT="BGK", relaxationTime=0.55, forcingSchemeT="Guo",
                  forceT="Kolmogorov", forceAmplitude=(1e-6, 0.0, 0.0),
                  forceWaveLength=(n / 2.0, 1.0, 1.0), kolmogorovAxis=2, kolmogorovComponent=0,
                  globalLength=(n, n, n))
    return {st: InputDeck(storage=st, **common) for st in ("f64", "f32", "f16_shifted")}


def entropic_decks(n: int):
    common = dict(latticeT="D3Q27", collisionT="ELBM", relaxationTime=1.0 / (2 * 0.9995),
                  globalLength=(n, n, n), alphaSolver="residual", newtonTolerance=1e-12,
                  deviationThreshold=0.0)
    return {"f64": InputDeck(storage="f64", alphaGuess="previous", **common),
            "f32": InputDeck(storage="f32", alphaGuess="learned", **common)}


def run(study: str, n: int, steps: list[int]):
    try:
        import torch
    except ImportError:  # spectra on the host
        torch = None
    shape = (n, n, n)
    if study == "bgk":
        decks = bgk_decks(n)
        rho, u = fields.perturbed_rest(shape, 3, 1e-4, seed=1)
    else:
        decks = entropic_decks(n)
        rho, u = fields.taylor_green(shape, u0=0.05)
        u = u + fields.solenoidal_shell(shape, 8.0, 10.0, 1e-3, seed=2)
    lats = {}
    for st, deck in decks.items():
        lat = Lattice(deck)
        if deck.alphaGuess == "learned":
            lat.set_alpha_model(alpha_model.load_model(alpha_model.default_model_path()))
        lat.init_equilibrium(rho, u)
        lats[st] = lat
    done = 0
    try:
        for target in sorted(steps):
            t0 = time.perf_counter()
            out = {}
            for st, lat in lats.items():
                lat.step(target - done, store=True)
                out[st] = lat.fields()
            done = target
            for st in out:
                if st == "f64":
                    continue
                line = {"study": study, "grid": n, "storage": st, "step": target,
                        **_errors(out["f64"], out[st], shape, torch),
                        "seconds": round(time.perf_counter() - t0, 1)}
                print(json.dumps(line), flush=True)
    finally:
        for lat in lats.values():
            lat.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["bgk", "entropic"])
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--steps", type=int, nargs="+", default=[500, 1000, 2000])
    a = ap.parse_args()
    run(a.study, a.grid, a.steps)


if __name__ == "__main__":
    main()
