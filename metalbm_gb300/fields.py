"""Initial fields for the benchmark workloads, generated on the host.

Random values come from a counter-based generator keyed by
(seed, component, global node index), so the same node gets the same value
whatever the array layout or process that builds it. The global node index
follows the reference's node order (Domain.h:88-91): (x*Ly + y)*Lz + z, with
z the contiguous axis.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea, Flood 2014), vectorised on uint64."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, component: int, index: np.ndarray) -> np.ndarray:
    """U[0,1) doubles for the given global node indices (53 random bits each)."""
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) * np.uint64(0xD1B54A32D192ED03)
               + np.uint64(component) * np.uint64(0x8CB92BA72F3D8DD7)
               + index.astype(np.uint64))
    r = _splitmix64(_splitmix64(key))
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def node_index(shape: tuple[int, int, int]) -> np.ndarray:
    lx, ly, lz = shape
    return np.arange(lx * ly * lz, dtype=np.uint64)


def perturbed_rest(shape, dims: int, amplitude: float, seed: int, rho0: float = 1.0,
                   rho_amplitude: float = 0.0):
    """rho = rho0 (+ optional uniform perturbation), u_d ~ U[-a, a] i.i.d.

    The fluid state of the bandwidth workloads: rho0 = 1, u uniform in
    [-1e-4, 1e-4] per component (seeds 0 and 1).
    Returns rho [V] and u [D, V] in reference node order.
    """
    idx = node_index(shape)
    u = np.stack([amplitude * (2.0 * uniform(seed, 1 + d, idx) - 1.0) for d in range(dims)])
    rho = np.full(idx.size, rho0)
    if rho_amplitude:
        rho = rho + rho_amplitude * (2.0 * uniform(seed, 0, idx) - 1.0)
    return rho, u


def taylor_green(shape, u0: float = 0.05, rho0: float = 1.0):
    """Taylor-Green vortex on [0, 2pi)^3 with c_s^2 = 1/3.

    u = U0 sin x cos y cos z, v = -U0 cos x sin y cos z, w = 0,
    p = rho0 U0^2 / 16 (cos 2x + cos 2y)(cos 2z + 2), rho = rho0 + 3 p.
    """
    lx, ly, lz = shape
    x = 2 * np.pi * np.arange(lx) / lx
    y = 2 * np.pi * np.arange(ly) / ly
    z = 2 * np.pi * np.arange(lz) / lz
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    ux = u0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    uy = -u0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    uz = np.zeros_like(ux)
    p = rho0 * u0 * u0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    rho = rho0 + 3.0 * p
    return rho.reshape(-1), np.stack([ux.reshape(-1), uy.reshape(-1), uz.reshape(-1)])


def solenoidal_shell(shape, kmin: float, kmax: float, amplitude: float, seed: int):
    """Random-phase divergence-free velocity on the wavenumber shell kmin<=|k|<=kmax.

    Each Fourier mode in the shell gets a random complex vector (counter-based
    draws keyed by the mode's index), projected orthogonal to k; the field is
    the real inverse FFT, scaled so that the largest |u| equals ``amplitude``.
    Returns u [3, V] in reference node order.
    """
    lx, ly, lz = shape
    kx = np.fft.fftfreq(lx, 1.0 / lx)
    ky = np.fft.fftfreq(ly, 1.0 / ly)
    kz = np.fft.rfftfreq(lz, 1.0 / lz)
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    shell = (k2 >= kmin * kmin) & (k2 <= kmax * kmax)
    idx = np.arange(KX.size, dtype=np.uint64).reshape(KX.shape)
    uh = []
    for d in range(3):
        re = 2.0 * uniform(seed, 10 + 2 * d, idx) - 1.0
        im = 2.0 * uniform(seed, 11 + 2 * d, idx) - 1.0
        uh.append(np.where(shell, re + 1j * im, 0.0))
    kk = np.where(k2 == 0, 1.0, k2)
    kdotu = (KX * uh[0] + KY * uh[1] + KZ * uh[2]) / kk
    uh = [uh[0] - KX * kdotu, uh[1] - KY * kdotu, uh[2] - KZ * kdotu]
    u = np.stack([np.fft.irfftn(c, s=(lx, ly, lz)) for c in uh])
    peak = np.sqrt((u ** 2).sum(axis=0)).max()
    if peak > 0:
        u *= amplitude / peak
    return u.reshape(3, -1)
