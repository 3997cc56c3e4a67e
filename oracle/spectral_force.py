"""Restatement of the reference's spectral forces, with numpy's FFT.

TEST INFRASTRUCTURE ONLY: the oracle the GPU force fields are checked
against; never imported by the product.

What is restated (reference file:line), per the code's evident intent:

* wavenumbers of the r2c half spectrum: k_d = i_d if i_d <= L_d/2 else
  i_d - L_d (integer wavenumbers, no 2 pi / L), the last axis 0..L/2
  (Force.h:339-347, Transformer.h:147-150);
* shell: kMin^2 <= |k|^2 <= kMax^2 (Force.h:386);
* ConstantShell (Force.h:294-431): a real spectrum equal to the amplitude on
  the shell, 2D - 3 components (one stream function in 2-D, a vector
  potential in 3-D), made solenoidal by MakeIncompressible
  (Transformer.h:298-401): the curl i k x T in 3-D (Transformer.h:207-272),
  (i k_y psi, -i k_x psi) in 2-D; then the backward transform divided by the
  node count (Transformer.h:98-108);
* EnergyRemoval (Force.h:434-572): F_d = -A_d P_shell(rho u_d), the momentum
  of the stored fields filtered to the shell; alone it takes forceAmplitude
  and forcekMin / forcekMax like every force (Algorithm.h:90-91);
* Turbulent2D (Force.h:575-622): ConstantShell(forceAmplitude, forcekMin,
  forcekMax) + EnergyRemoval(removalForceAmplitude, removalForcekMin,
  removalForcekMax).

Not restated: in 3-D the reference's Hermitian-partner writes on the
k_y = k_z = 0 row index y = L_y instead of 0 (Force.h:358-371, 481-494), so
they land one row off, and for x = 1 past the end of the component's
spectrum (into the next component's k = 0 mode, or past the array for the
last component). That is undefined behaviour and leaves the k_z = 0 plane
non-Hermitian, whose c2r transform FFTW does not define; the restatement
keeps every spectrum Hermitian. The shells must stay below the Nyquist
wavenumber (2 kMax < min L_d), so no shell mode is its own partner.

All functions return float64 arrays [D, V] in dense node order
(index (x*Ly + y)*Lz + z).
"""
from __future__ import annotations

import numpy as np


def _grid(shape, D):
    return tuple(shape[:D])


def wavenumbers(shape, D):
    """Integer wavenumbers of the rfftn half spectrum, broadcastable arrays."""
    g = _grid(shape, D)
    ks = []
    for d, n in enumerate(g):
        if d == D - 1:
            k = np.arange(n // 2 + 1)
        else:
            i = np.arange(n)
            k = np.where(i <= n // 2, i, i - n)
        sh = [1] * D
        sh[d] = k.size
        ks.append(k.reshape(sh).astype(np.float64))
    return ks


def shell_mask(shape, D, kmin, kmax):
    ks = wavenumbers(shape, D)
    k2 = sum(k * k for k in ks)
    return (k2 >= kmin * kmin) & (k2 <= kmax * kmax)


def _irfft(spec, shape, D):
    g = _grid(shape, D)
    return np.fft.irfftn(spec, s=g, axes=tuple(range(D))).reshape(-1)


def _rfft(x, shape, D):
    g = _grid(shape, D)
    return np.fft.rfftn(x.reshape(g), axes=tuple(range(D)))


def check_shell(shape, D, kmax):
    if 2 * kmax >= min(_grid(shape, D)):
        raise ValueError("the shell must stay below the Nyquist wavenumber (2 kMax < min L)")


def constant_shell_field(shape, D, amplitude, kmin, kmax):
    """ConstantShell: curl of the shell spectrum, divided by the node count."""
    check_shell(shape, D, kmax)
    m = shell_mask(shape, D, kmin, kmax).astype(np.float64)
    ks = wavenumbers(shape, D)
    if D == 2:
        psi = amplitude[0] * m
        spec = [1j * ks[1] * psi, -1j * ks[0] * psi]
    else:
        T = [amplitude[d] * m for d in range(3)]
        kx, ky, kz = ks
        spec = [1j * (ky * T[2] - kz * T[1]), 1j * (kz * T[0] - kx * T[2]),
                1j * (kx * T[1] - ky * T[0])]
    return np.stack([_irfft(np.broadcast_to(s, m.shape), shape, D) for s in spec])


def energy_removal_field(rho, u, shape, D, amplitude, kmin, kmax):
    """EnergyRemoval: -A_d times the shell-filtered momentum rho u_d."""
    check_shell(shape, D, kmax)
    m = shell_mask(shape, D, kmin, kmax)
    rho = np.asarray(rho, dtype=np.float64).reshape(-1)
    u = np.asarray(u, dtype=np.float64).reshape(D, -1)
    out = []
    for d in range(D):
        M = _rfft(rho * u[d], shape, D)
        out.append(_irfft(np.where(m, -amplitude[d] * M, 0.0), shape, D))
    return np.stack(out)


def turbulent_field(rho, u, shape, D, amplitude, kmin, kmax, removal_amplitude, removal_kmin,
                    removal_kmax):
    """Turbulent2D: injection (ConstantShell) plus removal (EnergyRemoval)."""
    return (constant_shell_field(shape, D, amplitude, kmin, kmax)
            + energy_removal_field(rho, u, shape, D, removal_amplitude, removal_kmin,
                                   removal_kmax))
