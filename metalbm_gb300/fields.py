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
    Built by broadcasting separable factors (no full-size coordinate grids).
    """
    lx, ly, lz = shape
    x = 2 * np.pi * np.arange(lx) / lx
    y = 2 * np.pi * np.arange(ly) / ly
    z = 2 * np.pi * np.arange(lz) / lz
    sx, cx = np.sin(x)[:, None, None], np.cos(x)[:, None, None]
    sy, cy = np.sin(y)[None, :, None], np.cos(y)[None, :, None]
    cz = np.cos(z)[None, None, :]
    u = np.empty((3, lx, ly, lz))
    u[0] = u0 * (sx * cy) * cz
    u[1] = -u0 * (cx * sy) * cz
    u[2] = 0.0
    c2 = (np.cos(2 * x)[:, None, None] + np.cos(2 * y)[None, :, None])
    rho = rho0 + 3.0 * (rho0 * u0 * u0 / 16.0) * c2 * (np.cos(2 * z)[None, None, :] + 2.0)
    return rho.reshape(-1), u.reshape(3, -1)


def solenoidal_shell(shape, kmin: float, kmax: float, amplitude: float, seed: int):
    """Random-phase divergence-free velocity on the wavenumber shell kmin<=|k|<=kmax.

    Each Fourier mode in the shell gets a random complex vector (counter-based
    draws keyed by the mode's index in the half-spectrum array), projected
    orthogonal to k; the field is the real inverse FFT, scaled so that the
    largest |u| equals ``amplitude``. Returns u [3, V] in reference node order.
    """
    lx, ly, lz = shape
    kx = np.fft.fftfreq(lx, 1.0 / lx)
    ky = np.fft.fftfreq(ly, 1.0 / ly)
    kz = np.fft.rfftfreq(lz, 1.0 / lz)
    nz = kz.size
    # shell modes only: |k| <= kmax bounds every component
    sel = [np.nonzero(np.abs(k) <= kmax)[0] for k in (kx, ky, kz)]
    I, J, K = np.meshgrid(*sel, indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    KX, KY, KZ = kx[I], ky[J], kz[K]
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    m = (k2 >= kmin * kmin) & (k2 <= kmax * kmax)
    I, J, K, KX, KY, KZ, k2 = I[m], J[m], K[m], KX[m], KY[m], KZ[m], k2[m]
    idx = ((I.astype(np.int64) * ly + J) * nz + K).astype(np.uint64)
    c = []
    for d in range(3):
        re = 2.0 * uniform(seed, 10 + 2 * d, idx) - 1.0
        im = 2.0 * uniform(seed, 11 + 2 * d, idx) - 1.0
        c.append(re + 1j * im)
    kdotu = (KX * c[0] + KY * c[1] + KZ * c[2]) / k2
    c = [c[0] - KX * kdotu, c[1] - KY * kdotu, c[2] - KZ * kdotu]
    u = np.empty((3, lx, ly, lz))
    for d in range(3):
        spec = np.zeros((lx, ly, nz), np.complex128)
        spec[I, J, K] = c[d]
        u[d] = np.fft.irfftn(spec, s=(lx, ly, lz), axes=(0, 1, 2))
    peak = np.sqrt((u ** 2).sum(axis=0)).max()
    if peak > 0:
        u *= amplitude / peak
    return u.reshape(3, -1)


def reference_initial_fields(shape, dims: int, density_type: str = "Homogeneous",
                             density_value: float = 1.0, velocity_type: str = "Homogeneous",
                             velocity_vector=(0.0, 0.0, 0.0)):
    """The reference's initial fields (initDensity / initVelocity,
    Initialize.h:19-68): density `density_value` everywhere, or for "Peak"
    three times that value at the single node
    ((Lx - 1) 0.4, (Ly - 1) 0.3, (Lz - 1) 0.2) (each truncated to an
    integer); velocity `velocity_vector` (its first `dims` components)
    everywhere. The reference's other velocity types (Perturbated, Wave,
    Decay) have no implementation there: it prints an error and keeps the
    homogeneous field, and so does this function."""
    lx, ly, lz = shape
    V = lx * ly * lz
    rho = np.full(V, float(density_value))
    if density_type == "Peak":
        cx, cy, cz = int((lx - 1) * 0.4), int((ly - 1) * 0.3), int((lz - 1) * 0.2)
        rho[(cx * ly + cy) * lz + cz] = 3.0 * float(density_value)
    elif density_type != "Homogeneous":
        raise ValueError(f"unknown initDensityT {density_type!r}")
    if velocity_type not in ("Homogeneous", "Perturbated", "Wave", "Decay"):
        raise ValueError(f"unknown initVelocityT {velocity_type!r}")
    u = np.empty((dims, V))
    for d in range(dims):
        u[d] = float(velocity_vector[d])
    return rho, u
