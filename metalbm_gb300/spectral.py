"""Spectral diagnostics of stored fields: vorticity, enstrophy, shell spectra.

Restates the reference's FFTW-based analyses for fields read back with
mlbm_get_fields (dense node order, [D][V]):

* Forward transforms are unnormalised real-to-complex transforms over the
  whole lattice; backward transforms divide by the volume V
  (Transformer.h:38-112).
* Wavenumbers are the signed integers k_d = i_d if i_d <= L_d/2 else i_d - L_d
  (Transformer.h:146-151, AnalysisList.h:140-148); no 2 pi / L factor.
* Curl (Transformer.h:118-187 in 2D, 189-295 in 3D): omega_hat = i k x u_hat,
  brought back with the normalised backward transform, then divided by V once
  more by Curl::normalize (Transformer.h:181-187, 285-294), which the reference's
  Routine calls after every evaluation (Routine.h:102-104, 128-131). In 2D the
  reference keeps only the real part of omega_hat (its imaginary part is
  multiplied by 0, Transformer.h:160-164). `reference=True` reproduces all of
  this; `reference=False` gives the textbook vorticity of a field sampled on
  [0, 2pi)^D (i k x u_hat with the integer wavenumbers, which are the
  wavenumbers of that domain, and the one normalisation of the inverse
  transform; for a lattice of unit spacing multiply component d's derivative
  by 2 pi / L_d instead).
* Shell energy spectrum (Analysis.h:122-177, AnalysisList.h:135-171): for each
  half-spectrum mode, 0.5 * sum_d |u_hat_d|^2 on the k_last = 0 plane and
  sum_d |u_hat_d|^2 elsewhere, added to shell floor(|k|) for
  floor(|k|) < max(L)/2 (FourierDomain.h:77-79), then divided by V.
* Total enstrophy (Analysis.h:68-98): (1/V) sum 1/2 |omega|^2.

Backend: numpy by default; pass torch CUDA tensors to run the transforms with
torch.fft (cuFFT) on the GPU.
"""
from __future__ import annotations

import numpy as np


def _xp(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return torch
    except ImportError:
        pass
    return np


def _wavenumbers(shape, xp, like):
    ks = []
    dims = len(shape)
    for d, L in enumerate(shape):
        n = L // 2 + 1 if d == dims - 1 else L
        i = np.arange(n)
        k = np.where(i <= L // 2, i, i - L).astype(np.float64)
        if xp is np:
            ks.append(k)
        else:
            ks.append(xp.tensor(k, dtype=xp.float64, device=like.device))
    grids = [None] * dims
    for d in range(dims):
        sh = [1] * dims
        sh[d] = -1
        grids[d] = ks[d].reshape(sh)
    return grids


def _rfftn(a, xp, shape):
    if xp is np:
        return np.fft.rfftn(a.reshape(shape))
    return xp.fft.rfftn(a.reshape(shape))


def _irfftn(a, xp, shape):
    axes = tuple(range(len(shape)))
    if xp is np:
        return np.fft.irfftn(a, s=shape, axes=axes)
    return xp.fft.irfftn(a, s=shape, dim=axes)


def active_shape(shape):
    """(Lx, Ly) for 2-D lattices (Lz = 1), (Lx, Ly, Lz) otherwise."""
    return tuple(shape[:2]) if len(shape) == 3 and shape[2] == 1 else tuple(shape)


def vorticity(u, shape, reference: bool = True):
    """Vorticity of u [D, V]: [1, V] in 2-D, [3, V] in 3-D (dense order)."""
    xp = _xp(u)
    sh = active_shape(shape)
    D = len(sh)
    V = int(np.prod(sh))
    uh = [_rfftn(u[d], xp, sh) for d in range(D)]
    k = _wavenumbers(sh, xp, u)
    if D == 2:
        w = 1j * (k[0] * uh[1] - k[1] * uh[0])
        if reference:
            w = w.real + 0j * w.real
        comps = [w]
    else:
        comps = [1j * (k[1] * uh[2] - k[2] * uh[1]),
                 1j * (k[2] * uh[0] - k[0] * uh[2]),
                 1j * (k[0] * uh[1] - k[1] * uh[0])]
    out = [_irfftn(c, xp, sh).reshape(-1) for c in comps]
    if reference:
        out = [o / V for o in out]
    return xp.stack(out)


def enstrophy(u, shape, reference: bool = True) -> float:
    """(1/V) sum 1/2 |omega|^2 (TotalEnstrophy, Analysis.h:68-98)."""
    w = vorticity(u, shape, reference)
    V = w.shape[1]
    return float((0.5 * (w * w).sum()) / V)


def energy(rho, u) -> float:
    """(1/V) sum 1/2 rho |u|^2 (TotalEnergy, Analysis.h:33-66)."""
    return float((0.5 * rho * (u * u).sum(0)).sum() / rho.shape[0])


def reference_shell_count(shape) -> int:
    """The reference's number of spectrum shells, gFD::maxWaveNumber()
    (FourierDomain.h:77-79): arrayMax(globalLength) / 2, whose recursion
    takes the minimum of the remaining lengths (Helpers.h:37-39), so
    max(L_x, min(L_y, L_z)) / 2 with L_z = 1 on 2-D lattices."""
    lx, ly, lz = (tuple(shape) + (1, 1))[:3]
    return max(lx, min(ly, lz)) // 2


def energy_spectrum(u, shape, reference: bool = True):
    """Shell-averaged energy spectrum E(k) (PowerSpectra, Analysis.h:122-177;
    AnalysisList.h:135-171, 194): k = 0 .. K - 1 with K the reference's shell
    count (`reference=True`, see reference_shell_count) or max(L) / 2."""
    xp = _xp(u)
    sh = active_shape(shape)
    D = len(sh)
    V = int(np.prod(sh))
    kmax = reference_shell_count(shape) if reference else max(sh) // 2
    k = _wavenumbers(sh, xp, u)
    kk = sum(c * c for c in k)
    knorm = xp.floor(xp.sqrt(kk)) if xp is not np else np.floor(np.sqrt(kk))
    e = 0.0
    for d in range(D):
        uh = _rfftn(u[d], xp, sh)
        e = e + uh.real ** 2 + uh.imag ** 2
    coef_shape = [1] * D
    coef_shape[-1] = -1
    nlast = sh[-1] // 2 + 1
    coef = np.ones(nlast)
    coef[0] = 0.5
    if xp is np:
        coef = coef.reshape(coef_shape)
        shells = np.broadcast_to(knorm, e.shape).astype(np.int64).ravel()
        w = (e * coef).ravel()
        keep = shells < kmax
        return np.bincount(shells[keep], weights=w[keep], minlength=kmax)[:kmax] / V
    coef = xp.tensor(coef, dtype=xp.float64, device=u.device).reshape(coef_shape)
    shells = knorm.expand(e.shape).to(xp.int64).reshape(-1)
    w = (e * coef).reshape(-1)
    keep = shells < kmax
    out = xp.zeros(kmax, dtype=xp.float64, device=u.device)
    out.index_add_(0, shells[keep], w[keep])
    return (out / V).cpu().numpy()
