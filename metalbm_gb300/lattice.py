"""Python host side of the drop-in: InputDeck, Lattice (one handle), Algorithm."""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import MlbmError

_LATTICES = {"D2Q9": capi.D2Q9, "D3Q19": capi.D3Q19, "D3Q27": capi.D3Q27,
             "D3Q15": capi.D3Q15, "D2Q13": capi.D2Q13, "D3Q33": capi.D3Q33}
# The entropic variants other than ELBM run as ELBM, as they do in the
# reference: their calculateAlpha overrides are never called from
# ELBM::calculateRelaxationTime (Collision.h:227-241).
_COLLISIONS = {"BGK": capi.BGK, "ELBM": capi.ELBM, "ForcedBNR_ELBM": capi.FORCED_BNR_ELBM,
               "Approached_ELBM": capi.APPROACHED_ELBM, "Malaspinas_ELBM": capi.MALASPINAS_ELBM,
               "Essentially1_ELBM": capi.ESSENTIALLY1_ELBM,
               "Essentially2_ELBM": capi.ESSENTIALLY2_ELBM, "ForcedNR_ELBM": capi.FORCED_NR_ELBM}
_UNSUPPORTED_COLLISIONS = {
    "ForcedNR_ELBM_Forcing": "subtracts the equilibrium from the pulled source populations in "
                             "place (Collision.h:757-775), so its result depends on the sweep "
                             "order",
    "GenericSRT": "abstract base of the SRT collisions", "GenericMRT": "abstract, no implementation"}
_FORCINGS = {"None": capi.FORCING_NONE, "Guo": capi.FORCING_GUO,
             "ShanChen": capi.FORCING_SHAN_CHEN,
             "ExactDifferenceMethod": capi.FORCING_EXACT_DIFFERENCE}
_FORCES = {"None": capi.FORCE_NONE, "Constant": capi.FORCE_CONSTANT,
           "Sinusoidal": capi.FORCE_SINUSOIDAL, "Kolmogorov": capi.FORCE_KOLMOGOROV,
           "ConstantShell": capi.FORCE_CONSTANT_SHELL, "EnergyRemoval": capi.FORCE_ENERGY_REMOVAL,
           "Turbulent2D": capi.FORCE_TURBULENT_2D}
_STORAGES = {"f64": capi.STORAGE_F64, "f32": capi.STORAGE_F32,
             "f16_shifted": capi.STORAGE_F16_SHIFTED}
_ALPHA = {"reference": capi.ALPHA_REFERENCE, "residual": capi.ALPHA_RESIDUAL}
_GUESS = {"previous": capi.GUESS_PREVIOUS, "two": capi.GUESS_TWO, "learned": capi.GUESS_LEARNED,
          "learned_everywhere": capi.GUESS_LEARNED_EVERYWHERE}
# default limit of Lattice.sync (a bounded poll; -1 waits without limit)
SYNC_TIMEOUT_MS = 600_000
Q_OF = {"D2Q9": 9, "D3Q19": 19, "D3Q27": 27, "D3Q15": 15, "D2Q13": 13, "D3Q33": 33}
D_OF = {"D2Q9": 2, "D3Q19": 3, "D3Q27": 3, "D3Q15": 3, "D2Q13": 2, "D3Q33": 3}


@dataclass
class InputDeck:
    """The Input.in parameters of the hot path (src/Input_prod.in:16-53),
    as a runtime configuration. Names follow the reference deck."""
    latticeT: str = "D2Q9"
    collisionT: str = "BGK"
    forcingSchemeT: str = "None"
    forceT: str = "None"
    relaxationTime: float = 0.7
    forceAmplitude: tuple = (0.0, 0.0, 0.0)
    forceWaveLength: tuple = (32.0, 32.0, 32.0)
    globalLength: tuple = (16, 16, 16)
    # Kolmogorov force: F[component] = A sin(2 pi x[axis] / lambda); the
    # reference is axis = 1 (y), component = 0 (x), Force.h:262-267.
    kolmogorovAxis: int = 1
    kolmogorovComponent: int = 0
    # initial fields (src/Input_prod.in:43-46, Initialize.h:19-68)
    initDensityT: str = "Homogeneous"
    initDensityValue: float = 1.0
    initVelocityT: str = "Homogeneous"
    initVelocityVector: tuple = (0.0, 0.0, 0.0)
    # spectral forces (src/Input_prod_3d.in:50-58): integer wavenumber shells
    forcekMin: int = 1
    forcekMax: int = 2
    removalForceAmplitude: tuple = (1e-6, 1e-6, 1e-6)
    removalForcekMin: int = 1
    removalForcekMax: int = 2
    # GB300 build options
    storage: str = "f64"
    alphaSolver: str = "reference"
    alphaGuess: str = "previous"
    newtonTolerance: float = 1e-8
    newtonMaxIterations: int = 50
    # cap of the residual solver's bisection-Newton (0: newtonMaxIterations)
    bisectionMaxIterations: int = 0
    # FP64 BGK arithmetic: "reference" (the reference's order, bit-identical)
    # or "fixed" (fixed-point moments and equilibrium on the integer pipe)
    fp64Arithmetic: str = "reference"
    deviationThreshold: float = 1e-3
    device: int = 0

    def __post_init__(self):
        self.forceAmplitude = tuple(self.forceAmplitude)
        self.forceWaveLength = tuple(self.forceWaveLength)
        self.globalLength = tuple(self.globalLength)
        self.removalForceAmplitude = tuple(self.removalForceAmplitude)
        self.initVelocityVector = tuple(self.initVelocityVector)

    @classmethod
    def from_reference_deck(cls, source, lengths=None, **overrides) -> "InputDeck":
        """An InputDeck from a reference deck (`src/Input_*.in`: a C++ header
        of `constexpr <type> <name> = <value>;` definitions), as text or a
        path. The hot path's parameters are taken over (lattice, collision,
        forcing, force and their amplitudes / wavelengths / shells, relaxation
        time, initial fields, lengths); lengths given as compile-time macros
        (GLOBAL_LENGTH_X ...) come from `lengths`. Choices this library does
        not implement raise ValueError: a non-Pull algorithm and an
        equilibrium other than TruncationMa3 (`Incompressible`, named by
        several shipped decks, is not an EquilibriumType of Options.h:31, so
        those decks do not compile in the reference either)."""
        import re
        from pathlib import Path
        if isinstance(source, Path):
            text = source.read_text()
        else:
            text = str(source)
            # a short single-line string without definitions names a file
            if ("constexpr" not in text and "\n" not in text and len(text) < 4096
                    and Path(text).is_file()):
                text = Path(text).read_text()
        defs = {}
        for line in text.splitlines():
            line = line.split("//")[0]
            m = re.match(r"\s*constexpr\s+[\w:<>]+(?:\s+int)?\s+(\w+)\s*=\s*(.+?);", line)
            if m:
                defs[m.group(1)] = m.group(2).strip()

        if not defs:
            raise ValueError("no `constexpr <type> <name> = <value>;` definitions in the deck")

        def enum(name):
            return defs[name].split("::")[-1]

        def vec(name):
            # MathVector<...>{{a, b, c}}: the numbers between the innermost braces
            inner = re.findall(r"\{([^{}]*)\}", defs[name])
            body = inner[-1] if inner else defs[name]
            try:
                return tuple(float(v) for v in body.split(",") if v.strip())
            except ValueError:
                raise ValueError(f"{name} = {defs[name]}: not a vector of numbers") from None

        if "algorithmT" in defs and enum("algorithmT") != "Pull":
            raise ValueError(f"algorithmT {enum('algorithmT')}: only the pull algorithm is built")
        if "equilibriumT" in defs and enum("equilibriumT") != "TruncationMa3":
            raise ValueError(f"equilibriumT {enum('equilibriumT')}: only TruncationMa3 is built "
                             "(Options.h:31 has no Incompressible)")
        kw = {}
        for key in ("latticeT", "collisionT", "forcingSchemeT", "forceT", "initDensityT",
                    "initVelocityT"):
            if key in defs:
                kw[key] = enum(key)
        for key in ("relaxationTime", "initDensityValue"):
            if key in defs:
                kw[key] = float(defs[key])
        for key in ("forcekMin", "forcekMax", "removalForcekMin", "removalForcekMax"):
            if key in defs:
                kw[key] = int(defs[key])
        for key in ("forceAmplitude", "forceWaveLength", "removalForceAmplitude",
                    "initVelocityVector"):
            if key in defs:
                kw[key] = vec(key)
        length = []
        for d, key in enumerate(("globalLengthX", "globalLengthY", "globalLengthZ")):
            v = defs.get(key, "1")
            if re.fullmatch(r"\d+", v):
                length.append(int(v))
            elif lengths is not None:
                length.append(int(lengths[d]))
            else:
                raise ValueError(f"{key} = {v}: give the lengths (lengths=(Lx, Ly, Lz))")
        kw["globalLength"] = tuple(length)
        kw.update(overrides)
        return cls(**kw)

    @property
    def Q(self) -> int:
        return Q_OF[self.latticeT]

    @property
    def D(self) -> int:
        return D_OF[self.latticeT]

    @property
    def shape(self) -> tuple[int, int, int]:
        lx, ly, lz = self.globalLength
        return (lx, ly, 1 if self.D == 2 else lz)

    def to_c(self) -> capi.Config:
        c = capi.Config()
        capi.load().mlbm_config_init(ct.byref(c))
        c.lattice = _LATTICES[self.latticeT]
        if self.collisionT in _UNSUPPORTED_COLLISIONS:
            raise ValueError(f"collisionT {self.collisionT!r} is not supported: "
                             f"{_UNSUPPORTED_COLLISIONS[self.collisionT]}")
        c.collision = _COLLISIONS[self.collisionT]
        c.forcing_scheme = _FORCINGS[self.forcingSchemeT]
        c.force = _FORCES[self.forceT]
        c.relaxation_time = float(self.relaxationTime)
        for d in range(3):
            c.force_amplitude[d] = float(self.forceAmplitude[d])
            c.force_wavelength[d] = float(self.forceWaveLength[d])
            c.length[d] = int(self.globalLength[d])
        c.kolmogorov_axis = int(self.kolmogorovAxis)
        c.kolmogorov_component = int(self.kolmogorovComponent)
        c.force_kmin, c.force_kmax = int(self.forcekMin), int(self.forcekMax)
        c.removal_kmin, c.removal_kmax = int(self.removalForcekMin), int(self.removalForcekMax)
        for d in range(3):
            c.removal_amplitude[d] = float(self.removalForceAmplitude[d])
        c.storage = _STORAGES[self.storage]
        c.alpha_mode = _ALPHA[self.alphaSolver]
        c.alpha_guess = _GUESS[self.alphaGuess]
        c.newton_tolerance = float(self.newtonTolerance)
        c.newton_max_iterations = int(self.newtonMaxIterations)
        c.bisection_max_iterations = int(self.bisectionMaxIterations)
        c.fp64_arithmetic = {"reference": 0, "fixed": 1}[self.fp64Arithmetic]
        c.deviation_threshold = float(self.deviationThreshold)
        c.device = int(self.device)
        return c


@dataclass
class MlpModel:
    """Weights of the alpha-guess MLP (n_in -> 32 -> 32 -> 1, tanh)."""
    n_in: int
    input_scale: np.ndarray
    w1: np.ndarray  # [32, n_in]
    b1: np.ndarray
    w2: np.ndarray  # [32, 32]
    b2: np.ndarray
    w3: np.ndarray  # [32]
    b3: float
    output_scale: float

    @staticmethod
    def init(n_in: int, input_scale, output_scale: float, seed: int = 0) -> "MlpModel":
        rng = np.random.default_rng(seed)
        h = capi.MLP_HIDDEN
        return MlpModel(n_in, np.asarray(input_scale, np.float32),
                        (rng.standard_normal((h, n_in)) / np.sqrt(n_in)).astype(np.float32),
                        np.zeros(h, np.float32),
                        (rng.standard_normal((h, h)) / np.sqrt(h)).astype(np.float32),
                        np.zeros(h, np.float32),
                        (rng.standard_normal(h) / np.sqrt(h)).astype(np.float32), 0.0,
                        float(output_scale))

    def to_c(self) -> capi.Mlp:
        m = capi.Mlp()
        m.n_in, m.n_hidden = self.n_in, capi.MLP_HIDDEN
        ct.memmove(m.input_scale, np.ascontiguousarray(self.input_scale, np.float32).ctypes.data,
                   4 * self.n_in)
        ct.memmove(m.w1, np.ascontiguousarray(self.w1, np.float32).ctypes.data, 4 * 32 * self.n_in)
        for name in ("b1", "b2", "w3"):
            ct.memmove(getattr(m, name), np.ascontiguousarray(getattr(self, name), np.float32)
                       .ctypes.data, 4 * 32)
        ct.memmove(m.w2, np.ascontiguousarray(self.w2, np.float32).ctypes.data, 4 * 32 * 32)
        m.b3 = float(self.b3)
        m.output_scale = float(self.output_scale)
        return m

    @staticmethod
    def from_c(m: capi.Mlp) -> "MlpModel":
        n = m.n_in
        arr = lambda a, k: np.ctypeslib.as_array(a)[:k].astype(np.float32).copy()  # noqa: E731
        return MlpModel(n, arr(m.input_scale, n), arr(m.w1, 32 * n).reshape(32, n),
                        arr(m.b1, 32), arr(m.w2, 1024).reshape(32, 32), arr(m.b2, 32),
                        arr(m.w3, 32), float(m.b3), float(m.output_scale))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_float))


class Lattice:
    """One periodic lattice on one GPU, driven through the C ABI."""

    def __init__(self, deck: InputDeck):
        self.deck = deck
        self._lib = capi.load()
        self.Q, self.D = deck.Q, deck.D
        self.shape = deck.shape
        self.V = int(np.prod(self.shape))
        cfg = deck.to_c()
        h = ct.c_void_p()
        rc = self._lib.mlbm_create(ct.byref(cfg), ct.byref(h))
        if rc != capi.OK:
            raise MlbmError(rc, self._lib.mlbm_last_error(None).decode())
        self._h = h

    # --- plumbing
    def _check(self, rc: int):
        if rc != capi.OK:
            raise MlbmError(rc, self._lib.mlbm_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mlbm_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        s = ct.c_void_p()
        self._check(self._lib.mlbm_get_stream(self._h, ct.byref(s)))
        return s.value or 0

    def set_stream(self, stream_ptr: int | None):
        self._check(self._lib.mlbm_set_stream(self._h, ct.c_void_p(stream_ptr or 0)))

    # --- state
    def initialize(self):
        """f = f_eq of the deck's initial fields (initDensity / initVelocity,
        then initDistribution, Initialize.h:19-116)."""
        from .fields import reference_initial_fields
        d = self.deck
        rho, u = reference_initial_fields(self.shape, self.D, d.initDensityT, d.initDensityValue,
                                          d.initVelocityT, d.initVelocityVector)
        self.init_equilibrium(rho, u)

    def init_equilibrium(self, rho: np.ndarray, u: np.ndarray, layout: int = capi.LAYOUT_DENSE):
        rho = np.ascontiguousarray(rho, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        self._check(self._lib.mlbm_init_equilibrium(self._h, _dptr(rho), _dptr(u), layout))

    def set_populations(self, f: np.ndarray, layout: int = capi.LAYOUT_DENSE):
        f = np.ascontiguousarray(f, np.float64)
        self._check(self._lib.mlbm_set_populations(self._h, _dptr(f), layout))

    def populations(self) -> np.ndarray:
        f = np.empty((self.Q, self.V))
        self._check(self._lib.mlbm_get_populations(self._h, _dptr(f), capi.LAYOUT_DENSE))
        return f

    def step(self, n: int = 1, store: bool = False, diagnostics: bool = False,
             samples: bool = False):
        flags = (capi.STEP_STORE_FIELDS if store else 0) | \
                (capi.STEP_DIAGNOSTICS if diagnostics else 0) | \
                (capi.STEP_LOG_SAMPLES if samples else 0)
        self._check(self._lib.mlbm_step(self._h, int(n), flags))

    def sync(self, timeout_ms: int = SYNC_TIMEOUT_MS):
        """Wait for the handle's stream (a bounded poll; MlbmError with
        ERR_TIMEOUT past `timeout_ms`, < 0 waits without limit), then check
        the device error word."""
        self._check(self._lib.mlbm_sync(self._h, int(timeout_ms)))

    def fields(self) -> dict[str, np.ndarray]:
        rho = np.empty(self.V)
        u = np.empty((self.D, self.V))
        alpha = np.empty(self.V)
        force = np.empty((self.D, self.V))
        self._check(self._lib.mlbm_get_fields(self._h, _dptr(rho), _dptr(u), _dptr(alpha),
                                              _dptr(force), capi.LAYOUT_DENSE))
        return {"rho": rho, "u": u, "alpha": alpha, "force": force}

    def spectral_diagnostics(self, vorticity: bool = True) -> dict:
        """The reference Routine's spectral analyses of the last stored fields,
        computed on the device (mlbm_get_spectral_diagnostics): vorticity
        [2D-3, V], energy, enstrophy and the shell spectrum."""
        n = ct.c_int()
        self._check(self._lib.mlbm_spectrum_shells(self._h, ct.byref(n)))
        w = np.empty((2 * self.D - 3, self.V)) if vorticity else None
        e, z = ct.c_double(), ct.c_double()
        spec = np.empty(n.value)
        self._check(self._lib.mlbm_get_spectral_diagnostics(
            self._h, _dptr(w) if w is not None else None, ct.byref(e), ct.byref(z),
            _dptr(spec) if n.value else None, capi.LAYOUT_DENSE))
        return {"vorticity": w, "energy": e.value, "enstrophy": z.value, "spectrum": spec}

    def diagnostics(self) -> dict:
        d = capi.Diag()
        self._check(self._lib.mlbm_get_diagnostics(self._h, ct.byref(d)))
        return d.as_dict()

    def alpha(self) -> np.ndarray:
        a = np.empty(self.V)
        self._check(self._lib.mlbm_get_alpha(self._h, _dptr(a), capi.LAYOUT_DENSE))
        return a

    def set_alpha(self, alpha: np.ndarray):
        a = np.ascontiguousarray(alpha, np.float64)
        self._check(self._lib.mlbm_set_alpha(self._h, _dptr(a), capi.LAYOUT_DENSE))

    # --- checkpoint / restart
    def save_checkpoint(self, path) -> None:
        """Populations (FP64, dense [Q][V]), the alpha field, the step count and
        the deck, in one .npz (the reference writes the distribution with its
        DistributionWriter, Writer.h:385-449, every backUpStep)."""
        import json
        from dataclasses import asdict
        d = self.diagnostics()
        np.savez(path, f=self.populations(), alpha=self.alpha(), step=np.int64(d["step"]),
                 deck=np.array(json.dumps(asdict(self.deck))))

    @staticmethod
    def from_checkpoint(path, **deck_overrides) -> "Lattice":
        """A lattice restored from save_checkpoint: populations and alpha as
        saved (the reference's restart reads f and re-initialises alpha to 2,
        Initialize.h:118-145; restoring alpha as well continues an entropic
        run exactly)."""
        import json
        z = np.load(path)
        deck = InputDeck(**{**json.loads(str(z["deck"])), **deck_overrides})
        lat = Lattice(deck)
        lat.set_populations(z["f"])
        lat.set_alpha(z["alpha"])
        return lat

    # --- sample logger and learned alpha
    def set_sample_nodes(self, nodes: np.ndarray):
        nodes = np.ascontiguousarray(nodes, np.int64)
        self._n_samples = len(nodes)
        self._check(self._lib.mlbm_set_sample_nodes(
            self._h, nodes.ctypes.data_as(ct.POINTER(ct.c_longlong)), len(nodes)))

    def samples(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = self._n_samples
        feat = np.empty((n, self.Q))
        alpha = np.empty(n)
        solved = np.empty(n, np.int32)
        self._check(self._lib.mlbm_get_samples(self._h, _dptr(feat), _dptr(alpha),
                                               solved.ctypes.data_as(ct.POINTER(ct.c_int))))
        return feat, alpha, solved

    def set_alpha_model(self, model: MlpModel):
        m = model.to_c()
        self._check(self._lib.mlbm_set_alpha_model(self._h, ct.byref(m)))

    def train_alpha_model(self, X: np.ndarray, y: np.ndarray, model: MlpModel, epochs: int = 10,
                          batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> tuple[MlpModel, float]:
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        cfg = capi.TrainCfg(epochs, batch, lr, 0.9, 0.999, 1e-8, seed, 0.0)
        m = model.to_c()
        self._check(self._lib.mlbm_train_alpha_model(self._h, _fptr(X), _fptr(y), len(y),
                                                     ct.byref(cfg), ct.byref(m)))
        return MlpModel.from_c(m), cfg.final_loss

    def alpha_model_gradient(self, model: MlpModel, X: np.ndarray, y: np.ndarray):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        m = model.to_c()
        g = capi.Mlp()
        loss = ct.c_float()
        self._check(self._lib.mlbm_alpha_model_gradient(self._h, ct.byref(m), _fptr(X), _fptr(y),
                                                        len(y), ct.byref(loss), ct.byref(g)))
        return float(loss.value), MlpModel.from_c(g)

    def alpha_model_predict(self, model: MlpModel, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        out = np.empty(len(X), np.float32)
        m = model.to_c()
        self._check(self._lib.mlbm_alpha_model_predict(self._h, ct.byref(m), _fptr(X), len(X),
                                                       _fptr(out)))
        return out


def kernel_launch_count() -> int:
    return int(capi.load().mlbm_kernel_launch_count())


class Algorithm:
    """metaLBM's Algorithm surface on the GPU lattice (Algorithm.h:23-29).

    ``iterate(iteration)`` runs one fused pull step (Algorithm.h:326-358);
    ``isStored`` makes that step store rho, u, alpha and F (Algorithm.h:67,
    150-194); ``unpack(local)`` / ``pack()`` move the populations in and out
    in the reference's padded local layout (Algorithm.h:132-147).
    """

    def __init__(self, lattice: Lattice):
        self.lattice = lattice
        self.isStored = False
        self._iteration = 0

    def iterate(self, iteration: int):
        self.lattice.step(1, store=self.isStored)
        self._iteration = iteration

    def unpack(self, local: np.ndarray):
        self.lattice.set_populations(local, capi.LAYOUT_REFERENCE)

    def pack(self, local: np.ndarray):
        f = np.ascontiguousarray(local, np.float64)
        self.lattice._check(self.lattice._lib.mlbm_get_populations(
            self.lattice.handle, _dptr(f), capi.LAYOUT_REFERENCE))
        local[...] = f
