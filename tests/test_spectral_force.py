"""Spectral forces (ConstantShell, EnergyRemoval, Turbulent2D; Force.h:294-626).

CPU: properties of the numpy restatement (oracle/spectral_force.py) and the
oracle's force-field mode. GPU: the C ABI's cuFFT force fields and the steps
driven by them against the oracle stepped with the restated fields.

Parity is unpinned against the reference itself: its spectral forces need
FFTW, and its 3-D partner writes on the k_y = k_z = 0 row are out of range
(see oracle/spectral_force.py). Tolerances: the force fields within
1e-13 max|F| (cuFFT and numpy's FFT round differently); populations within
1e-13 relative after the steps.
"""
import numpy as np
import pytest

from oracle import OracleConfig, OraclePort
from oracle import spectral_force as sf

TOL_FIELD = 1e-13
TOL_F = 1e-13


def _spec(F, shape, D):
    return np.stack([np.fft.rfftn(F[d].reshape(shape[:D])) for d in range(D)])


@pytest.mark.parametrize("D,shape", [(2, (24, 16, 1)), (3, (12, 10, 8))])
def test_constant_shell_is_solenoidal_and_on_the_shell(D, shape):
    F = sf.constant_shell_field(shape, D, (0.3, -0.2, 0.5), 1, 2)
    S = _spec(F, shape, D)
    ks = sf.wavenumbers(shape, D)
    div = sum(ks[d] * S[d] for d in range(D))
    assert np.abs(div).max() < 1e-12 * np.abs(S).max()
    off = ~sf.shell_mask(shape, D, 1, 2)
    assert np.abs(S[:, off]).max() < 1e-12 * np.abs(S).max()
    assert np.abs(F).max() > 0


@pytest.mark.parametrize("D,shape", [(2, (16, 20, 1)), (3, (10, 12, 8))])
def test_energy_removal_filters_the_momentum(D, shape):
    rng = np.random.default_rng(3)
    V = int(np.prod(shape[:D]))
    rho = 1 + 0.01 * rng.standard_normal(V)
    u = 0.02 * rng.standard_normal((D, V))
    A = (1e-3, 2e-3, 3e-3)
    F = sf.energy_removal_field(rho, u, shape, D, A, 1, 3)
    m = sf.shell_mask(shape, D, 1, 3)
    for d in range(D):
        M = np.fft.rfftn((rho * u[d]).reshape(shape[:D]))
        S = np.fft.rfftn(F[d].reshape(shape[:D]))
        assert np.allclose(S[m], -A[d] * M[m], rtol=0, atol=1e-13 * np.abs(M).max())
        assert np.abs(S[~m]).max() < 1e-13 * np.abs(M).max()


def test_shell_below_nyquist_is_required():
    with pytest.raises(ValueError):
        sf.constant_shell_field((8, 8, 8), 3, (1, 1, 1), 1, 4)


def test_oracle_field_force_equals_tabulated_force():
    """The oracle's force-field mode (Force<Generic>::setForce) driven with the
    per-node force of a Kolmogorov run reproduces that run bit for bit."""
    from metalbm_gb300 import fields
    shape = (12, 10, 8)
    rho, u = fields.perturbed_rest(shape, 3, 0.02, seed=4, rho_amplitude=0.01)
    kw = dict(lattice="D3Q19", forcing="Guo", tau=0.6, size=shape)
    a = OraclePort(OracleConfig(force="Kolmogorov", amplitude=(1e-3, 0, 0),
                                wavelength=(5.0, 1, 1), **kw))
    a.init_equilibrium(rho, u)
    a.step(1)
    F = a.fields()["force"]
    a.step(4)
    b = OraclePort(OracleConfig(force="Field", **kw))
    b.init_equilibrium(rho, u)
    b.set_force_field(F)
    b.step(5)
    assert np.array_equal(a.populations(), b.populations())


def _deck(lattice, force, shape, **kw):
    from metalbm_gb300 import InputDeck
    return InputDeck(latticeT=lattice, forcingSchemeT=kw.pop("forcing", "Guo"), forceT=force,
                     relaxationTime=kw.pop("tau", 0.6), globalLength=shape, **kw)


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape,forcing", [("D2Q9", (32, 24, 1), "Guo"),
                                                   ("D3Q19", (16, 12, 10), "Guo"),
                                                   ("D3Q27", (12, 16, 10), "ExactDifferenceMethod")])
def test_constant_shell_matches_oracle(lattice, shape, forcing):
    """ConstantShell (the 3-D production deck's force, Input_prod_3d.in:47-53):
    the force field and 8 steps against the oracle driven by the restated field."""
    from metalbm_gb300 import Lattice, fields
    D = 2 if lattice.startswith("D2") else 3
    A = (1e-3, -2e-3, 1.5e-3)
    rho, u = fields.perturbed_rest(shape, D, 0.02, seed=6, rho_amplitude=0.01)
    deck = _deck(lattice, "ConstantShell", shape, forcing=forcing, forceAmplitude=A,
                 forcekMin=1, forcekMax=3)
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        lat.step(8, store=True)
        f, fl = lat.populations(), lat.fields()
    Fref = sf.constant_shell_field(shape, D, A, 1, 3)
    assert np.abs(fl["force"] - Fref).max() <= TOL_FIELD * np.abs(Fref).max()
    port = OraclePort(OracleConfig(lattice=lattice, forcing=forcing, force="Field", tau=0.6,
                                   size=shape))
    port.init_equilibrium(rho, u)
    port.set_force_field(Fref)
    port.step(8)
    assert _rel(f, port.populations()) <= TOL_F


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape,force,rkmax,store_every",
                         [("D3Q19", (16, 12, 10), "EnergyRemoval", 3, 1),
                          ("D2Q9", (32, 24, 1), "Turbulent2D", 3, 1),
                          ("D3Q27", (12, 10, 16), "Turbulent2D", 3, 1),
                          ("D3Q19", (16, 14, 14), "EnergyRemoval", 6, 1),
                          ("D2Q9", (32, 24, 1), "Turbulent2D", 7, 1),
                          ("D3Q19", (16, 12, 10), "Turbulent2D", 2, 3)])
def test_time_dependent_spectral_force_matches_oracle(lattice, shape, force, rkmax, store_every):
    """EnergyRemoval / Turbulent2D: before every step the force comes from the
    last stored fields (Algorithm.h:338, Force.h:442-463), so between stores it
    does not change. Removal shells up to k = 5 take the separable partial
    transforms, larger ones cuFFT. Against the oracle with the restated field
    set before each step from its last stored fields."""
    from metalbm_gb300 import Lattice, fields
    D = 2 if lattice.startswith("D2") else 3
    A, RA = (2e-4, -1e-4, 3e-4), (0.05, 0.08, 0.03)
    rho, u = fields.perturbed_rest(shape, D, 0.03, seed=7, rho_amplitude=0.01)
    if force == "EnergyRemoval":  # alone it takes the force parameters (Algorithm.h:90-91)
        deck = _deck(lattice, force, shape, forceAmplitude=RA, forcekMin=1, forcekMax=rkmax)
    else:
        deck = _deck(lattice, force, shape, forceAmplitude=A, forcekMin=2, forcekMax=4,
                     removalForceAmplitude=RA, removalForcekMin=1, removalForcekMax=rkmax)
    steps = 6
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        for _ in range(steps // store_every):
            lat.step(store_every, store=True)
        f, fl = lat.populations(), lat.fields()
    port = OraclePort(OracleConfig(lattice=lattice, forcing="Guo", force="Field", tau=0.6,
                                   size=shape))
    port.init_equilibrium(rho, u)
    r, v = rho, u
    for _ in range(steps // store_every):
        if force == "EnergyRemoval":
            F = sf.energy_removal_field(r, v, shape, D, RA, 1, rkmax)
        else:
            F = sf.turbulent_field(r, v, shape, D, A, 2, 4, RA, 1, rkmax)
        port.set_force_field(F)
        port.step(store_every)
        pf = port.fields()
        r, v = pf["rho"], pf["u"]
    assert np.abs(fl["force"] - pf["force"]).max() <= 1e-12 * np.abs(pf["force"]).max()
    assert _rel(f, port.populations()) <= TOL_F
    assert np.abs(pf["force"]).max() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("storage,tol", [("f32", 2e-4), ("f16_shifted", 5e-3)])
@pytest.mark.parametrize("lattice,collision,force", [("D3Q27", "BGK", "ConstantShell"),
                                                     ("D3Q19", "BGK", "Turbulent2D"),
                                                     ("D2Q9", "ELBM", "EnergyRemoval")])
def test_spectral_force_low_precision_storage(storage, tol, lattice, collision, force):
    """FP32 / FP16-shifted storage read a float copy of the force field; u
    tracks the FP64-storage run within the storage tolerances of the other
    forces (test_low_precision_storage_tracks_f64), and the stored force field
    (FP64, from the stored fields) is the same to rounding."""
    from metalbm_gb300 import Lattice, fields
    D = 2 if lattice.startswith("D2") else 3
    shape = (16, 12, 10) if D == 3 else (32, 24, 1)
    rho, u = fields.perturbed_rest(shape, D, 0.02, seed=4, rho_amplitude=0.005)
    out = {}
    for st in ("f64", storage):
        deck = _deck(lattice, force, shape, forceAmplitude=(1e-4, -5e-5, 2e-5), forcekMin=1,
                     forcekMax=3, removalForceAmplitude=(0.05, 0.05, 0.05), storage=st,
                     collisionT=collision, tau=0.6 if collision == "BGK" else 0.52)
        with Lattice(deck) as lat:
            lat.init_equilibrium(rho, u)
            for _ in range(4):
                lat.step(5, store=True)
            out[st] = lat.fields()
    assert _rel(out[storage]["u"], out["f64"]["u"]) <= tol
    assert _rel(out[storage]["force"], out["f64"]["force"]) <= tol
