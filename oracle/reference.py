"""Runner for the reference metaLBM binaries built by oracle/build_ref.py.

Test infrastructure only; usable where the reference sources exist (the
golden-vector generator and the CPU timing on the machine that holds them).
Nothing the GPU tests, smoke() or bench.py run needs it.
"""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np

from .build_ref import CASES, OUT, compile_case

_Q = {"D2Q9": 9, "D3Q19": 19, "D3Q27": 27, "D3Q15": 15, "D2Q13": 13, "D3Q33": 33}
_D = {"D2Q9": 2, "D3Q19": 3, "D3Q27": 3, "D3Q15": 3, "D2Q13": 2, "D3Q33": 3}


def run_reference(case: str, rho: np.ndarray, u: np.ndarray, steps: int) -> dict:
    """Run reference case ``case`` from f = f_eq(rho, u) for ``steps`` steps.

    rho: [V]; u: [D, V] in dense reference node order. Returns f [Q, V], rho,
    u (hydrodynamic), alpha, force, the loop's wall seconds, and the
    reference's spectral analyses of the stored fields (vorticity, energy,
    enstrophy, spectrum).
    """
    c = CASES[case]
    exe = compile_case(case, c)
    Q, D = _Q[c.lattice], _D[c.lattice]
    lx, ly, lz = c.size
    if D == 2:
        lz = 1
    V = lx * ly * lz
    inp = np.concatenate([np.asarray(rho, np.float64).reshape(V),
                          np.asarray(u, np.float64).reshape(D * V)])
    with tempfile.TemporaryDirectory() as td:
        fi, fo = Path(td) / "in.bin", Path(td) / "out.bin"
        inp.tofile(fi)
        subprocess.run([str(exe), str(fi), str(fo), str(int(steps))], check=True,
                       cwd=str(OUT / case), capture_output=True)
        out = np.fromfile(fo, dtype=np.float64)
        fa = Path(str(fo) + ".analysis")
        an = np.fromfile(fa, dtype=np.float64) if fa.exists() else None
    o = 0

    def take(n):
        nonlocal o
        r = out[o:o + n]
        o += n
        return r

    f = take(Q * V).reshape(Q, V)
    rho_o = take(V)
    u_o = take(D * V).reshape(D, V)
    alpha = take(V)
    force = take(D * V).reshape(D, V)
    seconds = float(take(1)[0])
    res = {"f": f, "rho": rho_o, "u": u_o, "alpha": alpha, "force": force,
           "seconds": seconds}
    if an is not None:
        # the reference's spectral analyses of the stored fields (harness):
        # vorticity [2D-3, V], energy, enstrophy, energy spectrum [maxWaveNumber]
        nv = (2 * D - 3) * V
        res["vorticity"] = an[:nv].reshape(2 * D - 3, V)
        res["energy"], res["enstrophy"] = float(an[nv]), float(an[nv + 1])
        K = int(an[nv + 2])
        res["spectrum"] = an[nv + 3:nv + 3 + K]
    return res
