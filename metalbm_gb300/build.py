"""Build libmlbm.so in-tree with nvcc for sm_103a (GB300).

Each .cu file in csrc/ is compiled in parallel to an object in _build/ and
linked into metalbm_gb300/libmlbm.so. step_f64.cu is compiled with
-fmad=false so the FP64 kernels keep the reference's separately rounded
multiplies and adds (bit-identical BGK results); everything else may fuse.
ptxas resource usage (registers, spills, shared memory) goes to
_build/ptxas.log.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmlbm.so"
ROUTINE = PKG / "routine_gpu"   # C++ Routine-shaped driver on include/mlbm/Algorithm_gpu.h
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-Xptxas", "-v", f"-I{INCLUDE}", f"-I{CSRC}"]
PER_FILE = {"step_f64.cu": ["-fmad=false"], "step_f64x.cu": ["-fmad=false"]}


def units() -> list[tuple[Path, list[str], str]]:
    """(source, extra flags, object stem): the step kernels are compiled once
    per lattice (and storage format, and for the low-precision step forcing
    scheme) so the units build in parallel."""
    out = []
    for src in sorted(CSRC.glob("*.cu")):
        extra = PER_FILE.get(src.name, [])
        if src.name == "step_f64.cu":  # six lattices; one forcing scheme a unit
            out += [(src, extra + [f"-DMLBM_LAT={l}", f"-DMLBM_FS={fs}"], f"{src.stem}_L{l}_F{fs}")
                    for l in range(6) for fs in range(4)]
        elif src.name == "step_f64x.cu":  # D2Q9, D3Q19, D3Q27, D3Q15
            out += [(src, extra + [f"-DMLBM_LAT={l}"], f"{src.stem}_L{l}") for l in range(4)]
        elif src.name == "step_lowp.cu":  # D2Q9, D3Q19, D3Q27, D3Q15; one forcing scheme a unit
            out += [(src, extra + [f"-DMLBM_LAT={l}", f"-DMLBM_ST={st}", f"-DMLBM_FS={fs}"],
                     f"{src.stem}_L{l}_S{st}_F{fs}")
                    for l in range(4) for st in (1, 2) for fs in range(4)]
        else:
            out.append((src, extra, src.stem))
    return out


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise FileNotFoundError("nvcc not found")
    return exe


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        sorted(INCLUDE.glob("mlbm/*.h")) + sorted((PKG / "cpp").glob("*.cpp")) + [Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists() or not ROUTINE.exists():
        return False
    t = min(LIB.stat().st_mtime, ROUTINE.stat().st_mtime)
    return all(p.stat().st_mtime < t for p in _deps())


def build_routine() -> Path:
    """The C++ host driver, linked against libmlbm.so (rpath $ORIGIN)."""
    tmp = ROUTINE.with_name(f"routine_gpu.{os.getpid()}.tmp")
    cmd = ["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", str(PKG / "cpp" / "routine_gpu.cpp"),
           f"-L{PKG}", "-lmlbm", "-Wl,-rpath,$ORIGIN", "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building routine_gpu failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, ROUTINE)
    return ROUTINE


def _compile(unit) -> tuple[Path, str]:
    src, extra, stem = unit
    obj = BUILD / (stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr[-6000:]}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    todo = units()
    # longest units first: the D3Q27 low-precision steps (the entropic
    # kernels) and the D3Q33 / D3Q27 FP64 steps, then the other steps, the rest
    def cost(u):
        src, extra, _ = u
        if src.name == "step_lowp.cu":
            return (0 if "-DMLBM_LAT=2" in extra else 1, "-DMLBM_ST=2" in extra)
        if src.name == "step_f64.cu":
            return (0 if ("-DMLBM_LAT=5" in extra or "-DMLBM_LAT=2" in extra) else 1, True)
        return (2 if src.name.startswith("step_") else 3, False)
    todo.sort(key=cost)
    with cf.ThreadPoolExecutor(max(1, min(len(todo), os.cpu_count() or 1))) as ex:
        results = list(ex.map(_compile, todo))
    (BUILD / "ptxas.log").write_text("\n".join(log for _, log in results))
    tmp = LIB.with_suffix(f".so.{os.getpid()}.tmp")
    # cuFFT: the plain forward/backward transforms of the spectral forces
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *[str(o) for o, _ in results],
           "-Xcompiler", "-fPIC", "-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    build_routine()
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
