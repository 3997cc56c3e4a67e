"""Host spectral diagnostics (restatement of the reference's FFTW analyses).

Pinned against the reference itself: every golden vector carries the
reference's vorticity, total energy, total enstrophy and shell energy
spectrum of its stored fields (its Curl / TotalEnergy / TotalEnstrophy /
PowerSpectra run by the oracle harness with the DFT stand-in for FFTW).
"""
import json

import numpy as np
import pytest

from metalbm_gb300 import spectral
from metalbm_gb300.fields import taylor_green

from conftest import GOLDEN

GOLDEN_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def _golden(case):
    z = np.load(GOLDEN / f"{case}.npz")
    meta = json.loads(str(z["meta"]))
    D = 2 if meta["lattice"].startswith("D2") else 3
    lx, ly, lz = meta["size"]
    return z, (lx, ly, 1 if D == 2 else lz), D


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_analyses_match_reference(case):
    """Reference-mode vorticity (with its 2-D real-part-only curl and extra
    1/V), enstrophy, energy and shell spectrum of the reference's stored
    fields equal the reference's own analyses to rounding (FFT against the
    oracle's DFT): 1e-13 relative."""
    z, shape, D = _golden(case)
    w = spectral.vorticity(z["u"], shape, reference=True)
    assert np.abs(w - z["vorticity"]).max() <= 1e-13 * np.abs(z["vorticity"]).max()
    assert abs(spectral.enstrophy(z["u"], shape, reference=True) - float(z["enstrophy"])) <= \
        1e-13 * float(z["enstrophy"])
    assert abs(spectral.energy(z["rho"], z["u"]) - float(z["energy"])) <= 1e-13 * float(z["energy"])
    sp = np.asarray(spectral.energy_spectrum(z["u"], shape, reference=True))
    ref = z["spectrum"]
    assert sp.shape == ref.shape
    assert np.abs(sp - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["d2q9_bgk_guo_kolmogorov", "d3q19_bgk_guo_kolmogorov",
                                  "d3q27_elbm_none_none"])
def test_analyses_on_the_gpu_match_reference(case):
    """The same analyses on the device (cuFFT through torch) from the GPU
    step's stored fields, and the step's fused energy reduction, against the
    reference's analyses of its own run."""
    import torch
    from metalbm_gb300 import InputDeck, Lattice
    z, shape, D = _golden(case)
    meta = json.loads(str(z["meta"]))
    deck = InputDeck(latticeT=meta["lattice"], collisionT=meta["collision"],
                     forcingSchemeT=meta["forcing"], forceT=meta["force"],
                     relaxationTime=meta["tau"], forceAmplitude=tuple(meta["amp"]),
                     forceWaveLength=tuple(meta["wavelength"]), globalLength=tuple(meta["size"]))
    with Lattice(deck) as lat:
        lat.init_equilibrium(z["rho0"], z["u0"])
        lat.step(meta["steps"], store=True, diagnostics=True)
        fl, d = lat.fields(), lat.diagnostics()
    u = torch.from_numpy(fl["u"]).cuda()
    w = spectral.vorticity(u, shape, reference=True)
    w = w.cpu().numpy() if hasattr(w, "cpu") else np.asarray(w)
    tol = 1e-13 if meta["collision"] == "BGK" else 1e-11
    assert np.abs(w - z["vorticity"]).max() <= tol * np.abs(z["vorticity"]).max()
    sp = spectral.energy_spectrum(u, shape, reference=True)
    sp = sp.cpu().numpy() if hasattr(sp, "cpu") else np.asarray(sp)
    assert np.abs(sp - z["spectrum"]).max() <= tol * np.abs(z["spectrum"]).max()
    assert abs(d["energy"] - float(z["energy"])) <= tol * float(z["energy"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_library_analyses_match_reference(case):
    """The library's own analyses through the C ABI
    (mlbm_get_spectral_diagnostics: cuFFT transforms and the library's curl,
    shell and reduction kernels) of the GPU step's stored fields against the
    reference's Curl / TotalEnergy / TotalEnstrophy / PowerSpectra of its own
    run: 1e-13 where the fields are bit-identical (BGK with tabulated forces),
    1e-12 with the spectral forces (fields equal to 1e-13), 1e-11 for the
    entropic runs (fields equal to 1e-12)."""
    from metalbm_gb300 import InputDeck, Lattice
    z, shape, D = _golden(case)
    meta = json.loads(str(z["meta"]))
    spectral_force = meta["force"] in ("ConstantShell", "EnergyRemoval", "Turbulent2D")
    deck = InputDeck(latticeT=meta["lattice"], collisionT=meta["collision"],
                     forcingSchemeT=meta["forcing"], forceT=meta["force"],
                     relaxationTime=meta["tau"], forceAmplitude=tuple(meta["amp"]),
                     forceWaveLength=tuple(meta["wavelength"]), globalLength=tuple(meta["size"]),
                     forcekMin=meta.get("kmin", 1), forcekMax=meta.get("kmax", 2),
                     removalForceAmplitude=tuple(meta.get("ramp", (0.0, 0.0, 0.0))),
                     removalForcekMin=meta.get("rkmin", 1), removalForcekMax=meta.get("rkmax", 2))
    with Lattice(deck) as lat:
        lat.init_equilibrium(z["rho0"], z["u0"])
        lat.step(meta["steps"], store=True)
        a = lat.spectral_diagnostics()
    tol = 1e-11 if meta["collision"] != "BGK" else (1e-12 if spectral_force else 1e-13)
    assert a["vorticity"].shape == z["vorticity"].shape
    assert np.abs(a["vorticity"] - z["vorticity"]).max() <= tol * np.abs(z["vorticity"]).max()
    assert abs(a["enstrophy"] - float(z["enstrophy"])) <= tol * float(z["enstrophy"])
    assert abs(a["energy"] - float(z["energy"])) <= tol * float(z["energy"])
    assert a["spectrum"].shape == z["spectrum"].shape
    assert np.abs(a["spectrum"] - z["spectrum"]).max() <= tol * np.abs(z["spectrum"]).max()


def test_vorticity_of_taylor_green():
    shape = (24, 20, 16)
    _, u = taylor_green(shape, u0=1.0)
    w = spectral.vorticity(u, shape, reference=False).reshape(3, *shape)
    x = 2 * np.pi * np.arange(shape[0]) / shape[0]
    y = 2 * np.pi * np.arange(shape[1]) / shape[1]
    z = 2 * np.pi * np.arange(shape[2]) / shape[2]
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    assert np.abs(w[0] + np.cos(X) * np.sin(Y) * np.sin(Z)).max() < 1e-12
    assert np.abs(w[1] + np.sin(X) * np.cos(Y) * np.sin(Z)).max() < 1e-12
    assert np.abs(w[2] - 2 * np.sin(X) * np.sin(Y) * np.cos(Z)).max() < 1e-12


def test_reference_curl_normalisation_and_units():
    """Reference mode: integer wavenumbers and an extra 1/V (Curl::normalize)."""
    shape = (16, 12, 8)
    _, u = taylor_green(shape, u0=1.0)
    V = np.prod(shape)
    ref = spectral.vorticity(u, shape, reference=True)
    phys = spectral.vorticity(u, shape, reference=False)
    # on this grid every component of the TG field has wavenumber 1 on each
    # axis, so k_integer = k_phys * L / (2 pi) differs per axis: check one axis
    # at a time through a single-mode field
    u1 = np.zeros_like(u)
    yy = np.tile(np.arange(shape[1])[None, :, None], (shape[0], 1, shape[2])).ravel()
    u1[0] = np.sin(2 * np.pi * 3 * yy / shape[1])
    w = spectral.vorticity(u1, shape, reference=True)
    # omega_z = -d u_x / d y with integer k: -3 cos(...) / V
    assert np.abs(w[2] + 3 * np.cos(2 * np.pi * 3 * yy / shape[1]) / V).max() < 1e-13
    assert ref.shape == phys.shape == (3, V)


def test_reference_2d_curl_keeps_real_part_only():
    shape = (16, 12, 1)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((2, 16 * 12))
    w = spectral.vorticity(u, shape, reference=True)
    uh = [np.fft.rfftn(u[d].reshape(16, 12)) for d in range(2)]
    kx = np.where(np.arange(16) <= 8, np.arange(16), np.arange(16) - 16)[:, None]
    ky = np.arange(7)[None, :]
    re = (1j * (kx * uh[1] - ky * uh[0])).real
    expect = np.fft.irfftn(re + 0j, s=(16, 12), axes=(0, 1)).ravel() / (16 * 12)
    assert np.abs(w[0] - expect).max() < 1e-14


def test_reference_shell_count_takes_the_min_of_the_rest():
    """The reference's maxWaveNumber: max(L_x, min(L_y, L_z)) / 2."""
    assert spectral.reference_shell_count((8, 10, 9)) == 4
    assert spectral.reference_shell_count((12, 10, 8)) == 6
    assert spectral.reference_shell_count((16, 20, 1)) == 8
    assert spectral.reference_shell_count((32, 32, 32)) == 16


def test_energy_spectrum_single_shell_and_parseval():
    shape = (32, 32, 32)
    V = np.prod(shape)
    yy = np.tile(np.arange(32)[None, :, None], (32, 1, 32)).ravel()
    u = np.zeros((3, V))
    u[0] = np.sin(2 * np.pi * 2 * yy / 32)
    E = spectral.energy_spectrum(u, shape)
    assert E.shape == (16,)
    assert np.argmax(E) == 2 and abs(E.sum() - 0.5 * (u ** 2).sum()) < 1e-9 * V
    _, tg = taylor_green(shape, u0=0.1)
    E = spectral.energy_spectrum(tg, shape)
    assert abs(E.sum() - 0.5 * (tg ** 2).sum()) < 1e-12 * V
    assert np.argmax(E) == 1  # |k| = sqrt(2) -> shell 1


def test_reference_initial_fields_known_answers():
    """initDensity / initVelocity (Initialize.h:19-68): the Peak node and the
    homogeneous velocity."""
    from metalbm_gb300.fields import reference_initial_fields
    rho, u = reference_initial_fields((20, 12, 1), 2, "Peak", 1.5, "Homogeneous", (0.01, -0.02, 0.0))
    peak = (int(19 * 0.4) * 12 + int(11 * 0.3)) * 1 + 0
    assert rho[peak] == 4.5 and np.count_nonzero(rho != 1.5) == 1
    assert (u[0] == 0.01).all() and (u[1] == -0.02).all() and u.shape == (2, 240)
    rho, u = reference_initial_fields((8, 6, 5), 3, "Peak")
    assert rho[(int(7 * 0.4) * 6 + int(5 * 0.3)) * 5 + int(4 * 0.2)] == 3.0
    with pytest.raises(ValueError):
        reference_initial_fields((4, 4, 4), 3, "Gaussian")
