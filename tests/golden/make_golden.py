"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference metaLBM CPU path (built from the reference headers by
oracle/build_ref.py, so it needs the reference sources and only runs where
they exist) on small seeded inputs and stores inputs and outputs per case:

    <case>.npz : rho0 [V], u0 [D,V]          inputs (f starts at f_eq(rho0,u0))
                 f [Q,V], rho, u, alpha, force   reference state after `steps`
                 vorticity [2D-3,V], energy, enstrophy, spectrum
                                                 its spectral analyses of those fields
                 meta (json: the case parameters, steps, seeds)

All arrays are float64 in dense reference node order (index (x*Ly+y)*Lz+z).

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from dataclasses import asdict
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from metalbm_gb300 import fields  # noqa: E402
from oracle.build_ref import CASES, build  # noqa: E402
from oracle.reference import run_reference  # noqa: E402

OUT = Path(__file__).resolve().parent
STEPS = 20


def case_inputs(name: str):
    """Seeded inputs: BGK cases get |u| ~ 2e-2, entropic cases ~ 5e-2 so the
    Newton solve is active on a good share of nodes."""
    c = CASES[name]
    dims = 2 if c.lattice.startswith("D2") else 3
    shape = (c.size[0], c.size[1], 1 if dims == 2 else c.size[2])
    if c.collision == "BGK":
        seed, amp, ramp = 7, 0.02, 0.01
    else:
        seed, amp, ramp = 9, 0.05, 0.02
    rho, u = fields.perturbed_rest(shape, dims, amp, seed=seed, rho_amplitude=ramp)
    return rho, u, {"seed": seed, "u_amplitude": amp, "rho_amplitude": ramp}


def main(only=None) -> None:
    names = [n for n in CASES if not n.startswith("time_") and (not only or n in only)]
    build(names)
    for name in names:
        rho, u, gen = case_inputs(name)
        ref = run_reference(name, rho, u, STEPS)
        meta = {"case": name, "steps": STEPS, "generator": gen, **asdict(CASES[name])}
        # with the reference's spectral analyses of the stored fields: vorticity,
        # total energy and enstrophy, shell energy spectrum (Analysis.h:33-177)
        np.savez_compressed(OUT / f"{name}.npz", rho0=rho, u0=u, f=ref["f"], rho=ref["rho"],
                            u=ref["u"], alpha=ref["alpha"], force=ref["force"],
                            vorticity=ref["vorticity"], energy=ref["energy"],
                            enstrophy=ref["enstrophy"], spectrum=ref["spectrum"],
                            meta=np.array(json.dumps(meta)))
        print(name, "alpha range", ref["alpha"].min(), ref["alpha"].max())


if __name__ == "__main__":
    main(sys.argv[1:] or None)
