"""Build recipe for the reference metaLBM CPU path used as a test oracle.

Test infrastructure only. Each case is compiled from the reference headers
where they lie (<reference root>/include/metaLBM, never copied; the root is
the environment variable MLBM_REFERENCE_ROOT), with our
own MPI/HDF5/FFTW stand-ins from oracle/ref_stub, the deck oracle/ref_deck.in
and the harness oracle/ref_harness.cpp. Outputs go to oracle/_ref/<case>/run
(git-ignored). The reference is a header-only template library whose every
choice (lattice, collision, forcing, force, relaxation time, grid size) is a
compile-time constant, so each case is its own binary.

Flags: -O2 -ffp-contract=off so that the oracle computes every multiply and
add as a separately rounded IEEE operation on both x86-64 and aarch64 (the
aarch64 compiler would otherwise fuse them into FMAs).

Usage: python oracle/build_ref.py [case ...]     (no case = all cases)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from dataclasses import dataclass
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_INCLUDE = Path(os.environ.get("MLBM_REFERENCE_ROOT", "/root/reference")) / "include"
OUT = HERE / "_ref"


@dataclass(frozen=True)
class RefCase:
    lattice: str          # D2Q9 | D3Q19 | D3Q27 | D3Q15 | D2Q13 | D3Q33
    collision: str        # BGK | ELBM | ForcedBNR_ELBM | Approached_ELBM | ... (CollisionType)
    forcing: str          # None | Guo | ShanChen | ExactDifferenceMethod
    force: str            # None | Constant | Sinusoidal | Kolmogorov | ConstantShell | ...
    tau: float
    amp: tuple[float, float, float]
    wavelength: tuple[float, float, float]
    size: tuple[int, int, int]
    # spectral-force shells: forcekMin/Max, removalForceAmplitude, removalForcekMin/Max
    kmin: int = 1
    kmax: int = 2
    ramp: tuple[float, float, float] = (0.0, 0.0, 0.0)
    rkmin: int = 1
    rkmax: int = 2


# Small cases for golden vectors (non-square, non-power-of-two grids to catch
# axis mix-ups) and the timing cases of the CPU baseline.
CASES: dict[str, RefCase] = {
    # D2Q9
    "d2q9_bgk_guo_kolmogorov": RefCase("D2Q9", "BGK", "Guo", "Kolmogorov", 0.6,
                                       (1e-3, 0.0, 0.0), (6.0, 1.0, 1.0), (20, 12, 1)),
    "d2q9_bgk_none_none": RefCase("D2Q9", "BGK", "None", "None", 0.8,
                                  (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (16, 10, 1)),
    "d2q9_bgk_shanchen_constant": RefCase("D2Q9", "BGK", "ShanChen", "Constant", 0.7,
                                          (2e-4, -1e-4, 0.0), (1.0, 1.0, 1.0), (14, 18, 1)),
    "d2q9_bgk_edm_sinusoidal": RefCase("D2Q9", "BGK", "ExactDifferenceMethod", "Sinusoidal",
                                       0.55, (1e-3, 5e-4, 0.0), (7.0, 9.0, 1.0), (21, 18, 1)),
    "d2q9_elbm_guo_kolmogorov": RefCase("D2Q9", "ELBM", "Guo", "Kolmogorov", 0.52,
                                        (1e-4, 0.0, 0.0), (8.0, 1.0, 1.0), (24, 16, 1)),
    # D3Q19
    "d3q19_bgk_guo_kolmogorov": RefCase("D3Q19", "BGK", "Guo", "Kolmogorov", 0.55,
                                        (1e-3, 0.0, 0.0), (5.0, 1.0, 1.0), (12, 10, 8)),
    "d3q19_bgk_edm_sinusoidal": RefCase("D3Q19", "BGK", "ExactDifferenceMethod", "Sinusoidal",
                                        0.9, (1e-3, 2e-3, -1e-3), (6.0, 5.0, 7.0), (9, 10, 7)),
    "d3q19_bgk_shanchen_constant": RefCase("D3Q19", "BGK", "ShanChen", "Constant", 0.65,
                                           (1e-4, 2e-4, 3e-4), (1.0, 1.0, 1.0), (8, 6, 10)),
    "d3q19_bgk_none_none": RefCase("D3Q19", "BGK", "None", "None", 0.6,
                                   (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (7, 9, 6)),
    # D3Q27
    "d3q27_bgk_guo_kolmogorov": RefCase("D3Q27", "BGK", "Guo", "Kolmogorov", 0.6,
                                        (1e-3, 0.0, 0.0), (4.0, 1.0, 1.0), (10, 8, 6)),
    "d3q27_bgk_guo_sinusoidal": RefCase("D3Q27", "BGK", "Guo", "Sinusoidal", 0.75,
                                        (1e-3, -2e-3, 1e-3), (5.0, 4.0, 6.0), (10, 8, 6)),
    "d3q27_elbm_none_none": RefCase("D3Q27", "ELBM", "None", "None", 0.500250125062531,
                                    (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q27_elbm_guo_kolmogorov": RefCase("D3Q27", "ELBM", "Guo", "Kolmogorov", 0.51,
                                         (1e-4, 0.0, 0.0), (5.0, 1.0, 1.0), (10, 10, 6)),
    "d3q27_forcedbnr_none_none": RefCase("D3Q27", "ForcedBNR_ELBM", "None", "None",
                                         0.500250125062531, (0.0, 0.0, 0.0),
                                         (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q19_elbm_edm_constant": RefCase("D3Q19", "ELBM", "ExactDifferenceMethod", "Constant",
                                       0.53, (1e-4, -1e-4, 2e-4), (1.0, 1.0, 1.0), (8, 9, 10)),
    # the other entropic collision types, same parameters as d3q27_elbm_none_none
    # (they inherit ELBM::calculateRelaxationTime, Collision.h:227-241)
    "d3q27_approached_none_none": RefCase("D3Q27", "Approached_ELBM", "None", "None",
                                          0.500250125062531, (0.0, 0.0, 0.0),
                                          (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q27_malaspinas_none_none": RefCase("D3Q27", "Malaspinas_ELBM", "None", "None",
                                          0.500250125062531, (0.0, 0.0, 0.0),
                                          (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q27_essentially1_none_none": RefCase("D3Q27", "Essentially1_ELBM", "None", "None",
                                            0.500250125062531, (0.0, 0.0, 0.0),
                                            (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q27_essentially2_none_none": RefCase("D3Q27", "Essentially2_ELBM", "None", "None",
                                            0.500250125062531, (0.0, 0.0, 0.0),
                                            (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q27_forcednr_none_none": RefCase("D3Q27", "ForcedNR_ELBM", "None", "None",
                                        0.500250125062531, (0.0, 0.0, 0.0),
                                        (1.0, 1.0, 1.0), (12, 10, 8)),
    # the other lattices of Lattice.h:213-533, 706-802 (D2Q13 and D3Q33 reach
    # two nodes away: halo 2)
    "d3q15_bgk_guo_kolmogorov": RefCase("D3Q15", "BGK", "Guo", "Kolmogorov", 0.57,
                                        (1e-3, 0.0, 0.0), (5.0, 1.0, 1.0), (12, 10, 8)),
    "d3q15_bgk_shanchen_constant": RefCase("D3Q15", "BGK", "ShanChen", "Constant", 0.7,
                                           (2e-4, -1e-4, 1e-4), (1.0, 1.0, 1.0), (9, 8, 10)),
    "d3q15_elbm_edm_sinusoidal": RefCase("D3Q15", "ELBM", "ExactDifferenceMethod", "Sinusoidal",
                                         0.51, (1e-4, -2e-4, 1e-4), (6.0, 5.0, 7.0), (10, 9, 8)),
    "d2q13_bgk_none_none": RefCase("D2Q13", "BGK", "None", "None", 0.8, (0.0, 0.0, 0.0),
                                   (1.0, 1.0, 1.0), (16, 20, 1)),
    "d2q13_bgk_guo_kolmogorov": RefCase("D2Q13", "BGK", "Guo", "Kolmogorov", 0.6,
                                        (1e-3, 0.0, 0.0), (6.0, 1.0, 1.0), (20, 12, 1)),
    "d2q13_bgk_edm_sinusoidal": RefCase("D2Q13", "BGK", "ExactDifferenceMethod", "Sinusoidal",
                                        0.75, (1e-3, -2e-3, 0.0), (7.0, 5.0, 1.0), (14, 10, 1)),
    "d2q13_elbm_guo_kolmogorov": RefCase("D2Q13", "ELBM", "Guo", "Kolmogorov", 0.52,
                                         (1e-4, 0.0, 0.0), (8.0, 1.0, 1.0), (24, 16, 1)),
    "d3q33_bgk_guo_kolmogorov": RefCase("D3Q33", "BGK", "Guo", "Kolmogorov", 0.58,
                                        (1e-3, 0.0, 0.0), (5.0, 1.0, 1.0), (12, 10, 8)),
    "d3q33_bgk_shanchen_constant": RefCase("D3Q33", "BGK", "ShanChen", "Constant", 0.66,
                                           (2e-4, 1e-4, -1e-4), (1.0, 1.0, 1.0), (8, 10, 9)),
    "d3q33_elbm_none_none": RefCase("D3Q33", "ELBM", "None", "None", 0.500250125062531,
                                    (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (12, 10, 8)),
    "d3q33_elbm_edm_constant": RefCase("D3Q33", "ELBM", "ExactDifferenceMethod", "Constant", 0.51,
                                       (1e-4, -2e-4, 1e-4), (1.0, 1.0, 1.0), (10, 9, 8)),
    "d3q15_bgk_edm_kolmogorov": RefCase("D3Q15", "BGK", "ExactDifferenceMethod", "Kolmogorov",
                                        0.62, (1e-3, 0.0, 0.0), (7.0, 1.0, 1.0), (9, 14, 8)),
    "d2q13_bgk_shanchen_constant": RefCase("D2Q13", "BGK", "ShanChen", "Constant", 0.68,
                                           (2e-4, -1e-4, 0.0), (1.0, 1.0, 1.0), (18, 14, 1)),
    # 2-D spectral forces (Force.h:294-626), with the DFT stand-in of
    # oracle/ref_stub/fftw3-mpi.h; well defined in 2-D (the 3-D partner writes
    # are out of range)
    "d2q9_bgk_guo_constantshell": RefCase("D2Q9", "BGK", "Guo", "ConstantShell", 0.6,
                                          (1e-3, -2e-3, 0.0), (1.0, 1.0, 1.0), (24, 16, 1),
                                          kmin=1, kmax=3),
    "d2q9_bgk_guo_energyremoval": RefCase("D2Q9", "BGK", "Guo", "EnergyRemoval", 0.6,
                                          (0.05, 0.08, 0.0), (1.0, 1.0, 1.0), (24, 16, 1),
                                          kmin=1, kmax=3),
    "d2q9_bgk_edm_turbulent2d": RefCase("D2Q9", "BGK", "ExactDifferenceMethod", "Turbulent2D",
                                        0.7, (2e-3, 1e-3, 0.0), (1.0, 1.0, 1.0), (20, 24, 1),
                                        kmin=2, kmax=4, ramp=(0.04, 0.03, 0.0), rkmin=1,
                                        rkmax=2),
    "d2q9_elbm_guo_turbulent2d": RefCase("D2Q9", "ELBM", "Guo", "Turbulent2D", 0.52,
                                         (1e-3, 0.0, 0.0), (1.0, 1.0, 1.0), (24, 20, 1),
                                         kmin=3, kmax=5, ramp=(0.05, 0.05, 0.0), rkmin=1,
                                         rkmax=2),
    # CPU-baseline timing cases (sizes of the benchmark workloads, run for a
    # bounded number of steps).
    "time_d3q19_bgk_guo_kolmogorov_128": RefCase("D3Q19", "BGK", "Guo", "Kolmogorov", 0.55,
                                                 (1e-6, 0.0, 0.0), (64.0, 1.0, 1.0),
                                                 (128, 128, 128)),
    "time_d3q27_elbm_none_64": RefCase("D3Q27", "ELBM", "None", "None", 0.500250125062531,
                                       (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (64, 64, 64)),
}


def _lit(v: float) -> str:
    return repr(float(v))


def compile_case(name: str, case: RefCase, harness: Path | None = None) -> Path:
    if not REF_INCLUDE.is_dir():
        raise FileNotFoundError(f"reference headers not found at {REF_INCLUDE}")
    out_dir = OUT / name
    out_dir.mkdir(parents=True, exist_ok=True)
    exe = out_dir / "run"
    stamp = out_dir / "cmd"  # the compile command of `exe`: a changed case rebuilds
    harness = harness or HERE / "ref_harness.cpp"
    sources = [harness, HERE / "ref_deck.in"] + sorted(HERE.glob("ref_stub/*.h"))
    defs = {
        "NPROCS": "1", "NTHREADS": "1", "USE_FFTW": "1",
        "GLOBAL_LENGTH_X": str(case.size[0]), "GLOBAL_LENGTH_Y": str(case.size[1]),
        "GLOBAL_LENGTH_Z": str(case.size[2]), "LBM_POSTFIX": f'"{name}"',
        "MLBM_LATTICE": case.lattice, "MLBM_COLLISION": case.collision,
        "MLBM_FORCING": case.forcing, "MLBM_FORCE": case.force,
        "MLBM_TAU": _lit(case.tau),
        "MLBM_AMP_X": _lit(case.amp[0]), "MLBM_AMP_Y": _lit(case.amp[1]),
        "MLBM_AMP_Z": _lit(case.amp[2]),
        "MLBM_WL_X": _lit(case.wavelength[0]), "MLBM_WL_Y": _lit(case.wavelength[1]),
        "MLBM_WL_Z": _lit(case.wavelength[2]),
        "MLBM_KMIN": str(case.kmin), "MLBM_KMAX": str(case.kmax),
        "MLBM_RAMP_X": _lit(case.ramp[0]), "MLBM_RAMP_Y": _lit(case.ramp[1]),
        "MLBM_RAMP_Z": _lit(case.ramp[2]),
        "MLBM_RKMIN": str(case.rkmin), "MLBM_RKMAX": str(case.rkmax),
    }
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-fpermissive", "-w",
           f"-I{HERE / 'ref_stub'}", f"-I{HERE}", f"-I{REF_INCLUDE / 'metaLBM'}",
           f"-I{REF_INCLUDE}"]
    if case.force in ("Constant", "Sinusoidal"):
        defs[f"MLBM_FORCE_IS_{case.force.upper()}"] = "1"
    cmd += [f"-D{k}={v}" for k, v in defs.items()]
    cmd += [str(harness), "-o", str(exe)]
    if (exe.exists() and stamp.exists() and stamp.read_text() == " ".join(cmd)
            and all(exe.stat().st_mtime > src.stat().st_mtime for src in sources)):
        return exe
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"building {name} failed:\n{res.stderr[-4000:]}")
    stamp.write_text(" ".join(cmd))
    return exe


def build_bisection(lattice: str = "D3Q27") -> Path:
    """oracle/_ref/bisection_<lattice>/run: the reference's
    Bisection_NewtonRaphsonSolver with its EntropicStepFunctor on given node
    data (oracle/ref_bisection.cpp), for the golden vectors of
    tests/golden/bisection/."""
    case = RefCase(lattice, "ELBM", "None", "None", 0.500250125062531, (0.0, 0.0, 0.0),
                   (1.0, 1.0, 1.0), (4, 4, 4) if lattice[1] == "3" else (4, 4, 1))
    return compile_case(f"bisection_{lattice.lower()}", case, HERE / "ref_bisection.cpp")


def build(names: list[str] | None = None, jobs: int | None = None) -> dict[str, Path]:
    names = list(CASES) if not names else names
    jobs = jobs or max(1, min(len(names), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = {n: ex.submit(compile_case, n, CASES[n]) for n in names}
        return {n: f.result() for n, f in futs.items()}


if __name__ == "__main__":
    built = build(sys.argv[1:] or None)
    for n, p in built.items():
        print(n, p)
