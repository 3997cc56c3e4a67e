"""ctypes binding of the C restatement oracle/mlbm_oracle.c (test infrastructure).

The C file is compiled with -O2 -ffp-contract=off so that its arithmetic is
the reference's, operation for operation, on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
import threading
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB_PATH = BUILD / "liboracle.so"

LATTICES = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2, "D3Q15": 3, "D2Q13": 4, "D3Q33": 5}
COLLISIONS = {"BGK": 0, "ELBM": 1}
FORCINGS = {"None": 0, "Guo": 1, "ShanChen": 2, "ExactDifferenceMethod": 3}
# "Field": the per-node force read from an array set with set_force_field
FORCES = {"None": 0, "Constant": 1, "Sinusoidal": 2, "Kolmogorov": 3, "Field": 4}
ALPHA_REFERENCE, ALPHA_RESIDUAL = 0, 1
GUESS_PREVIOUS, GUESS_TWO = 0, 1
_Q = {"D2Q9": 9, "D3Q19": 19, "D3Q27": 27, "D3Q15": 15, "D2Q13": 13, "D3Q33": 33}
_D = {"D2Q9": 2, "D3Q19": 3, "D3Q27": 3, "D3Q15": 3, "D2Q13": 2, "D3Q33": 3}

_lock = threading.Lock()


class _Cfg(ct.Structure):
    _fields_ = [("lattice", ct.c_int), ("collision", ct.c_int), ("forcing", ct.c_int),
                ("force", ct.c_int), ("tau", ct.c_double), ("amplitude", ct.c_double * 3),
                ("wavelength", ct.c_double * 3), ("kolmogorov_axis", ct.c_int),
                ("kolmogorov_component", ct.c_int), ("lx", ct.c_int), ("ly", ct.c_int),
                ("lz", ct.c_int), ("alpha_mode", ct.c_int), ("guess_mode", ct.c_int),
                ("newton_tolerance", ct.c_double), ("newton_max_iterations", ct.c_int),
                ("deviation_threshold", ct.c_double), ("threads", ct.c_int),
                ("bisection_max_iterations", ct.c_int), ("log_ulp_perturbation", ct.c_int),
                ("population_ulp_perturbation", ct.c_int)]


def build_port(force: bool = False) -> Path:
    """Compile oracle/mlbm_oracle.c into oracle/_build/liboracle.so."""
    src = [HERE / "mlbm_oracle.c", HERE / "mlbm_oracle.h"]
    with _lock:
        if (not force and LIB_PATH.exists()
                and all(LIB_PATH.stat().st_mtime > s.stat().st_mtime for s in src)):
            return LIB_PATH
        BUILD.mkdir(exist_ok=True)
        tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c99",
                        "-D_POSIX_C_SOURCE=200809L", str(src[0]), "-o", str(tmp), "-lm",
                        "-lpthread"], check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ct.CDLL(str(build_port()))
        dp = ct.POINTER(ct.c_double)
        lib.oracle_create.restype = ct.c_void_p
        lib.oracle_create.argtypes = [ct.POINTER(_Cfg)]
        lib.oracle_destroy.argtypes = [ct.c_void_p]
        lib.oracle_init_equilibrium.argtypes = [ct.c_void_p, dp, dp]
        lib.oracle_set_populations.argtypes = [ct.c_void_p, dp]
        lib.oracle_get_populations.argtypes = [ct.c_void_p, dp]
        lib.oracle_step.argtypes = [ct.c_void_p, ct.c_int, ct.c_int]
        lib.oracle_get_fields.argtypes = [ct.c_void_p, dp, dp, dp, dp]
        lib.oracle_set_force_field.argtypes = [ct.c_void_p, dp]
        lib.oracle_get_counters.argtypes = [ct.c_void_p] + [ct.POINTER(ct.c_longlong)] * 3
        lib.oracle_equilibrium.restype = ct.c_double
        lib.oracle_equilibrium.argtypes = [ct.c_int, ct.c_double, dp, ct.c_int]
        lib.oracle_lattice_tables.argtypes = [ct.c_int, dp, dp]
        lib.oracle_solve_alpha_nodes.argtypes = [ct.c_int, ct.c_double, ct.c_int, ct.c_int,
                                                 ct.c_long, dp, dp, dp, dp,
                                                 ct.POINTER(ct.c_int)]
        lib.oracle_fast_log.restype = ct.c_double
        lib.oracle_fast_log.argtypes = [ct.c_double]
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


def lattice_tables(lattice: str) -> tuple[np.ndarray, np.ndarray]:
    """(c[Q,3] as float64, w[Q]) in the reference's population order."""
    q = _Q[lattice]
    c = np.zeros(q * 3)
    w = np.zeros(q)
    _load().oracle_lattice_tables(LATTICES[lattice], _ptr(c), _ptr(w))
    return c.reshape(q, 3), w


@dataclass
class OracleConfig:
    lattice: str = "D2Q9"
    collision: str = "BGK"
    forcing: str = "None"
    force: str = "None"
    tau: float = 0.6
    amplitude: tuple = (0.0, 0.0, 0.0)
    wavelength: tuple = (1.0, 1.0, 1.0)
    kolmogorov_axis: int = 1
    kolmogorov_component: int = 0
    size: tuple = (16, 16, 1)
    alpha_mode: int = ALPHA_REFERENCE
    guess_mode: int = GUESS_PREVIOUS
    newton_tolerance: float = 1e-8
    newton_max_iterations: int = 50
    deviation_threshold: float = 1e-3
    threads: int = 1
    bisection_max_iterations: int = 0  # 0: the Newton cap
    log_ulp_perturbation: int = 0  # sensitivity tests: libm log moved by one ulp
    population_ulp_perturbation: int = 0  # sensitivity tests: BGK results moved by one ulp


class OraclePort:
    """One lattice on the host, advanced by the C restatement."""

    def __init__(self, cfg: OracleConfig):
        self.cfg = cfg
        self.Q, self.D = _Q[cfg.lattice], _D[cfg.lattice]
        lx, ly, lz = cfg.size
        if self.D == 2:
            lz = 1
        self.shape = (lx, ly, lz)
        self.V = lx * ly * lz
        c = _Cfg(LATTICES[cfg.lattice], COLLISIONS[cfg.collision], FORCINGS[cfg.forcing],
                 FORCES[cfg.force], cfg.tau, (ct.c_double * 3)(*cfg.amplitude),
                 (ct.c_double * 3)(*cfg.wavelength), cfg.kolmogorov_axis,
                 cfg.kolmogorov_component, lx, ly, lz, cfg.alpha_mode, cfg.guess_mode,
                 cfg.newton_tolerance, cfg.newton_max_iterations, cfg.deviation_threshold,
                 max(1, cfg.threads), int(cfg.bisection_max_iterations),
                 int(cfg.log_ulp_perturbation), int(cfg.population_ulp_perturbation))
        self._lib = _load()
        self._h = self._lib.oracle_create(ct.byref(c))
        if not self._h:
            raise MemoryError("oracle_create failed")

    def close(self):
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def init_equilibrium(self, rho: np.ndarray, u: np.ndarray):
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.V)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(self.D, self.V)
        self._lib.oracle_init_equilibrium(self._h, _ptr(rho), _ptr(u))

    def set_populations(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.Q * self.V)
        self._lib.oracle_set_populations(self._h, _ptr(f))

    def populations(self) -> np.ndarray:
        f = np.empty((self.Q, self.V))
        self._lib.oracle_get_populations(self._h, _ptr(f))
        return f

    def step(self, n: int, store_last: bool = True):
        self._lib.oracle_step(self._h, int(n), int(bool(store_last)))

    def set_force_field(self, force: np.ndarray):
        """Per-node force [D, V] for force "Field" (Force.h:36-45)."""
        force = np.ascontiguousarray(force, dtype=np.float64).reshape(self.D * self.V)
        self._lib.oracle_set_force_field(self._h, _ptr(force))

    def fields(self) -> dict[str, np.ndarray]:
        rho = np.empty(self.V)
        u = np.empty((self.D, self.V))
        alpha = np.empty(self.V)
        force = np.empty((self.D, self.V))
        self._lib.oracle_get_fields(self._h, _ptr(rho), _ptr(u), _ptr(alpha), _ptr(force))
        return {"rho": rho, "u": u, "alpha": alpha, "force": force}

    def counters(self) -> dict[str, int]:
        a, b, c = ct.c_longlong(), ct.c_longlong(), ct.c_longlong()
        self._lib.oracle_get_counters(self._h, ct.byref(a), ct.byref(b), ct.byref(c))
        return {"newton_iterations": a.value, "fallbacks": b.value, "bisections": c.value}


def equilibrium(lattice: str, rho: float, u, q: int) -> float:
    uu = np.zeros(3)
    uu[:len(u)] = u
    return _load().oracle_equilibrium(LATTICES[lattice], float(rho), _ptr(uu), int(q))


def fast_log(x: float) -> float:
    """The residual mode's FP64 logarithm (Tang's table-driven method)."""
    return _load().oracle_fast_log(float(x))


def solve_alpha_nodes(lattice: str, f: np.ndarray, fneq: np.ndarray, guess: np.ndarray,
                      tol: float = 1e-12, newton_maxit: int = 50, bisect_maxit: int = 50):
    """The residual-mode alpha solve on single nodes (f, f_neq: [n, Q]):
    (alpha [n], flags [n]: 1 limited, 2 bracketed solver ran, 4 alpha = 2)."""
    f = np.ascontiguousarray(f, np.float64)
    fneq = np.ascontiguousarray(fneq, np.float64)
    guess = np.ascontiguousarray(guess, np.float64)
    n = f.shape[0]
    alpha = np.empty(n)
    flags = np.empty(n, np.int32)
    _load().oracle_solve_alpha_nodes(LATTICES[lattice], float(tol), int(newton_maxit),
                                     int(bisect_maxit), n, _ptr(f), _ptr(fneq), _ptr(guess),
                                     _ptr(alpha), flags.ctypes.data_as(ct.POINTER(ct.c_int)))
    return alpha, flags
