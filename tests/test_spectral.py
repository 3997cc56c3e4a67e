"""Host spectral diagnostics (restatement of the reference's FFTW analyses)."""
import numpy as np

from metalbm_gb300 import spectral
from metalbm_gb300.fields import taylor_green


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
    expect = np.fft.irfftn(re + 0j, s=(16, 12)).ravel() / (16 * 12)
    assert np.abs(w[0] - expect).max() < 1e-14


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
