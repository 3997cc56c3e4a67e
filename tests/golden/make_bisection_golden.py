"""Golden vectors of the bracketed entropic alpha solver, from the reference.

The reference's Bisection_NewtonRaphsonSolver (EntropicStep.h:142-220), with
its own EntropicStepFunctor (EntropicStep.h:15-63), is run by the harness
oracle/ref_bisection.cpp (built from the reference headers by
oracle/build_ref.py, so this script only runs where the reference sources
exist) on node data of a D3Q27 Taylor-Green flow:

* populations: the oracle port's FP64 ELBM runs (tau = 0.50025) of three
  flows with growing deviations: Taylor-Green 12^3, U0 = 0.08, 4 steps;
  Taylor-Green 6^3, U0 = 0.12, 3 steps (under-resolved); a seeded random
  velocity field (|u| ~ 0.08, density +-0.03) on 8^3 after 2 steps; at every
  node the pulled populations f_q(x - c_q) and f_neq = f - f_eq(rho, u) (the
  reference equilibrium);
* only nodes with alpha_max >= 2 kept (the nodes that reach the solver), up
  to 100 drawn per flow (seed 3);
* the solver with tolerance 1e-12 and iterationMax 50, from [1, alpha_max].

Output tests/golden/bisection/d3q27_nodes.npz: f [n, 27], fneq [n, 27],
alpha_max [n], alpha [n] and converged [n] of the reference, meta (json).

Usage: python tests/golden/make_bisection_golden.py
"""
from __future__ import annotations

import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from metalbm_gb300 import fields  # noqa: E402
from oracle import OracleConfig, OraclePort, lattice_tables  # noqa: E402
from oracle.build_ref import build_bisection  # noqa: E402
from oracle.port import equilibrium  # noqa: E402

OUT = Path(__file__).resolve().parent / "bisection"
TOL, MAXIT = 1e-12, 50
PER_FLOW = 100


def node_data(shape, rho0, u0, steps, tau=0.50025):
    """Pulled populations and f_neq [V, 27] of the oracle port's state."""
    port = OraclePort(OracleConfig(lattice="D3Q27", collision="ELBM", tau=tau, size=shape,
                                   deviation_threshold=0.0))
    port.init_equilibrium(rho0, u0)
    port.step(steps)
    F = port.populations().reshape(27, *shape)
    c, w = lattice_tables("D3Q27")
    f = np.stack([np.roll(F[q], shift=tuple(int(v) for v in c[q]), axis=(0, 1, 2)).ravel()
                  for q in range(27)], axis=1)
    rho = f.sum(axis=1)
    u = (f @ c) / rho[:, None]
    feq = np.array([[equilibrium("D3Q27", rho[i], u[i], q) for q in range(27)]
                    for i in range(f.shape[0])])
    return f, f - feq


def flows():
    yield (12, 12, 12), fields.taylor_green((12, 12, 12), u0=0.08), 4
    yield (6, 6, 6), fields.taylor_green((6, 6, 6), u0=0.12), 3
    yield (8, 8, 8), fields.perturbed_rest((8, 8, 8), 3, 0.08, seed=4, rho_amplitude=0.03), 2


def alpha_max(f, fneq):
    """min(2.5, min over f_neq > 0 of f / f_neq) (Collision.h:305-326)."""
    ratio = np.where(fneq > 0, np.abs(f) / np.where(fneq > 0, fneq, 1.0), np.inf)
    return np.minimum(2.5, ratio.min(axis=1))


def main() -> None:
    exe = build_bisection("D3Q27")
    rng = np.random.default_rng(3)
    rows_f, rows_n = [], []
    for shape, (rho0, u0), steps in flows():
        f, fneq = node_data(shape, rho0, u0, steps)
        keep = np.flatnonzero(alpha_max(f, fneq) >= 2.0)
        pick = rng.choice(keep, size=min(PER_FLOW, keep.size), replace=False)
        rows_f.append(f[pick])
        rows_n.append(fneq[pick])
    f, fneq = np.concatenate(rows_f), np.concatenate(rows_n)
    amax = alpha_max(f, fneq)
    n = f.shape[0]
    rec = np.concatenate([f, fneq, amax[:, None], np.full((n, 1), 2.0)], axis=1)
    with tempfile.TemporaryDirectory() as td:
        fi, fo = Path(td) / "in.bin", Path(td) / "out.bin"
        np.concatenate([[float(n)], rec.ravel()]).tofile(fi)
        subprocess.run([str(exe), str(fi), str(fo), repr(TOL), str(MAXIT)], check=True)
        out = np.fromfile(fo).reshape(n, 2)
    meta = {"lattice": "D3Q27", "tolerance": TOL, "iteration_max": MAXIT, "per_flow": PER_FLOW,
            "flows": ["Taylor-Green 12^3 U0 0.08, 4 steps", "Taylor-Green 6^3 U0 0.12, 3 steps",
                      "random |u| 0.08, rho +-0.03, 8^3, seed 4, 2 steps"], "tau": 0.50025,
            "solver": "Bisection_NewtonRaphsonSolver (EntropicStep.h:142-220) on [1, alpha_max]"}
    OUT.mkdir(exist_ok=True)
    np.savez_compressed(OUT / "d3q27_nodes.npz", f=f, fneq=fneq, alpha_max=amax,
                        alpha=out[:, 0], converged=out[:, 1], meta=json.dumps(meta))
    print(f"{n} nodes, {int(out[:, 1].sum())} converged -> {OUT / 'd3q27_nodes.npz'}")


if __name__ == "__main__":
    main()
