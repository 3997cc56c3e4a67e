"""ctypes binding of the mlbm C ABI (include/mlbm/mlbm.h).

The library is the in-tree metalbm_gb300/libmlbm.so built by
metalbm_gb300/build.py. There is no fallback: if the library is missing or no
CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmlbm.so"

# status codes
OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_TIMEOUT, ERR_NUMERIC, ERR_STATE, ERR_NO_DEVICE = range(8)
# enums (Options.h:12-43)
D2Q9, D3Q19, D3Q27, D3Q15, D2Q13, D3Q33 = 0, 1, 2, 3, 4, 5
BGK, ELBM, FORCED_BNR_ELBM = 0, 1, 2
APPROACHED_ELBM, MALASPINAS_ELBM, ESSENTIALLY1_ELBM, ESSENTIALLY2_ELBM, FORCED_NR_ELBM = range(3, 8)
FORCING_NONE, FORCING_GUO, FORCING_SHAN_CHEN, FORCING_EXACT_DIFFERENCE = 0, 1, 2, 3
FORCE_NONE, FORCE_CONSTANT, FORCE_SINUSOIDAL, FORCE_KOLMOGOROV = 0, 1, 2, 3
FORCE_CONSTANT_SHELL, FORCE_ENERGY_REMOVAL, FORCE_TURBULENT_2D = 4, 5, 6
STORAGE_F64, STORAGE_F32, STORAGE_F16_SHIFTED = 0, 1, 2
ALPHA_REFERENCE, ALPHA_RESIDUAL = 0, 1
GUESS_PREVIOUS, GUESS_TWO, GUESS_LEARNED, GUESS_LEARNED_EVERYWHERE = 0, 1, 2, 3
LAYOUT_DENSE, LAYOUT_REFERENCE = 0, 1
STEP_STORE_FIELDS, STEP_DIAGNOSTICS, STEP_LOG_SAMPLES = 1, 2, 4
MLP_HIDDEN, MLP_MAX_IN = 32, 27

EXPORTS = [
    "mlbm_config_init", "mlbm_create", "mlbm_destroy", "mlbm_init_equilibrium",
    "mlbm_set_populations", "mlbm_get_populations", "mlbm_step", "mlbm_get_fields",
    "mlbm_get_diagnostics", "mlbm_sync", "mlbm_get_stream", "mlbm_set_stream",
    "mlbm_set_sample_nodes", "mlbm_get_samples", "mlbm_set_alpha_model",
    "mlbm_train_alpha_model", "mlbm_alpha_model_gradient", "mlbm_alpha_model_predict",
    "mlbm_last_error", "mlbm_kernel_launch_count", "mlbm_step_f64_noalloc",
    "mlbm_get_alpha", "mlbm_set_alpha", "mlbm_spectrum_shells", "mlbm_get_spectral_diagnostics",
]
TESTING_EXPORTS = ["mlbm_testing_fast_log", "mlbm_testing_entropy", "mlbm_testing_neq",
                   "mlbm_testing_alpha_solve", "mlbm_testing_step_in_place"]


class Config(ct.Structure):
    _fields_ = [("lattice", ct.c_int), ("collision", ct.c_int), ("forcing_scheme", ct.c_int),
                ("force", ct.c_int), ("relaxation_time", ct.c_double),
                ("force_amplitude", ct.c_double * 3), ("force_wavelength", ct.c_double * 3),
                ("kolmogorov_axis", ct.c_int), ("kolmogorov_component", ct.c_int),
                ("length", ct.c_int * 3), ("storage", ct.c_int), ("alpha_mode", ct.c_int),
                ("alpha_guess", ct.c_int), ("newton_tolerance", ct.c_double),
                ("newton_max_iterations", ct.c_int), ("deviation_threshold", ct.c_double),
                ("device", ct.c_int), ("force_kmin", ct.c_int), ("force_kmax", ct.c_int),
                ("removal_kmin", ct.c_int), ("removal_kmax", ct.c_int),
                ("removal_amplitude", ct.c_double * 3), ("bisection_max_iterations", ct.c_int),
                ("fp64_arithmetic", ct.c_int), ("reserved", ct.c_int * 2)]


class Diag(ct.Structure):
    _fields_ = [("step", ct.c_longlong), ("mass", ct.c_double), ("energy", ct.c_double),
                ("max_mach", ct.c_double), ("alpha_min", ct.c_double), ("alpha_max", ct.c_double),
                ("solved_nodes", ct.c_longlong), ("newton_iterations", ct.c_longlong),
                ("guess_hits", ct.c_longlong), ("bisection_nodes", ct.c_longlong),
                ("fallback_nodes", ct.c_longlong), ("limited_nodes", ct.c_longlong),
                ("shortcut_nodes", ct.c_longlong), ("error_word", ct.c_uint),
                ("reserved0", ct.c_uint), ("series_nodes", ct.c_longlong),
                ("learned_nodes", ct.c_longlong), ("reserved", ct.c_double * 4)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("reserved")}


class Mlp(ct.Structure):
    _fields_ = [("n_in", ct.c_int), ("n_hidden", ct.c_int),
                ("input_scale", ct.c_float * MLP_MAX_IN),
                ("w1", ct.c_float * (MLP_HIDDEN * MLP_MAX_IN)), ("b1", ct.c_float * MLP_HIDDEN),
                ("w2", ct.c_float * (MLP_HIDDEN * MLP_HIDDEN)), ("b2", ct.c_float * MLP_HIDDEN),
                ("w3", ct.c_float * MLP_HIDDEN), ("b3", ct.c_float),
                ("output_scale", ct.c_float)]


class TrainCfg(ct.Structure):
    _fields_ = [("epochs", ct.c_int), ("batch", ct.c_int), ("learning_rate", ct.c_float),
                ("beta1", ct.c_float), ("beta2", ct.c_float), ("eps", ct.c_float),
                ("seed", ct.c_ulonglong), ("final_loss", ct.c_float)]


_lib = None


def load(path: Path | str | None = None):
    """Load libmlbm.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} not built: run metalbm_gb300/build.py")
    lib = ct.CDLL(str(p))
    vp, dp, fp = ct.c_void_p, ct.POINTER(ct.c_double), ct.POINTER(ct.c_float)
    sig = {
        "mlbm_config_init": ([ct.POINTER(Config)], ct.c_int),
        "mlbm_create": ([ct.POINTER(Config), ct.POINTER(vp)], ct.c_int),
        "mlbm_destroy": ([vp], ct.c_int),
        "mlbm_init_equilibrium": ([vp, dp, dp, ct.c_int], ct.c_int),
        "mlbm_set_populations": ([vp, dp, ct.c_int], ct.c_int),
        "mlbm_get_populations": ([vp, dp, ct.c_int], ct.c_int),
        "mlbm_step": ([vp, ct.c_int, ct.c_uint], ct.c_int),
        "mlbm_get_fields": ([vp, dp, dp, dp, dp, ct.c_int], ct.c_int),
        "mlbm_get_diagnostics": ([vp, ct.POINTER(Diag)], ct.c_int),
        "mlbm_get_alpha": ([vp, dp, ct.c_int], ct.c_int),
        "mlbm_set_alpha": ([vp, dp, ct.c_int], ct.c_int),
        "mlbm_sync": ([vp, ct.c_int], ct.c_int),
        "mlbm_get_stream": ([vp, ct.POINTER(vp)], ct.c_int),
        "mlbm_set_stream": ([vp, vp], ct.c_int),
        "mlbm_set_sample_nodes": ([vp, ct.POINTER(ct.c_longlong), ct.c_longlong], ct.c_int),
        "mlbm_get_samples": ([vp, dp, dp, ct.POINTER(ct.c_int)], ct.c_int),
        "mlbm_set_alpha_model": ([vp, ct.POINTER(Mlp)], ct.c_int),
        "mlbm_train_alpha_model": ([vp, fp, fp, ct.c_longlong, ct.POINTER(TrainCfg),
                                    ct.POINTER(Mlp)], ct.c_int),
        "mlbm_alpha_model_gradient": ([vp, ct.POINTER(Mlp), fp, fp, ct.c_longlong, fp,
                                       ct.POINTER(Mlp)], ct.c_int),
        "mlbm_alpha_model_predict": ([vp, ct.POINTER(Mlp), fp, ct.c_longlong, fp], ct.c_int),
        "mlbm_last_error": ([vp], ct.c_char_p),
        "mlbm_kernel_launch_count": ([], ct.c_ulonglong),
        "mlbm_step_f64_noalloc": ([ct.POINTER(Config), vp, vp, vp, vp, vp, vp], ct.c_int),
        "mlbm_spectrum_shells": ([vp, ct.POINTER(ct.c_int)], ct.c_int),
        "mlbm_get_spectral_diagnostics": ([vp, dp, dp, dp, dp, ct.c_int], ct.c_int),
        "mlbm_testing_fast_log": ([dp, dp, ct.c_longlong], ct.c_int),
        "mlbm_testing_entropy": ([ct.c_int, fp, dp, ct.c_longlong, dp, ct.c_int, ct.c_int, dp,
                                  dp, ct.POINTER(ct.c_int)], ct.c_int),
        "mlbm_testing_neq": ([ct.c_int, fp, ct.c_longlong, ct.c_int, dp], ct.c_int),
        "mlbm_testing_alpha_solve": ([ct.c_int, ct.c_double, ct.c_int, ct.c_int, ct.c_longlong,
                                      dp, dp, dp, dp, ct.POINTER(ct.c_int)], ct.c_int),
        "mlbm_testing_step_in_place": ([vp], ct.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


class MlbmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"mlbm error {code}: {message}")
        self.code = code
