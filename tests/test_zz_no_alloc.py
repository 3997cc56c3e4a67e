"""The allocation-free FP64 BGK step (mlbm_step_f64_noalloc).

For callers that cannot allocate device memory: the entry point runs on the
caller's device buffers and keeps its diagnostics scratch in a static device
array. Checked through the C ABI against the handle-based step on the same
state, for two calls in a row (the second consumes the first's output, so
the shared scratch is reused). Collected last so that a failure here comes
after every other test has run.
"""
import ctypes as ct
import math

import numpy as np
import pytest


def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _sin_profiles(amp, lam, shape, D):
    """The Sinusoidal force's per-axis profiles A_d sin(i 2 pi / lambda_d),
    concatenated x, y(, z), as the caller passes them (Force.h:208-215)."""
    return np.concatenate([[amp[d] * math.sin(float(i * 2) * math.pi / lam[d])
                            for i in range(shape[d])] for d in range(D)])


def _call(lib, cfg, d_in, d_out, d_prof, d_diag, d_err, torch):
    from metalbm_gb300 import capi
    rc = lib.mlbm_step_f64_noalloc(
        ct.byref(cfg), ct.c_void_p(d_in.data_ptr()), ct.c_void_p(d_out.data_ptr()),
        ct.c_void_p(d_prof.data_ptr()) if d_prof is not None else None,
        ct.c_void_p(d_diag.data_ptr()), ct.c_void_p(d_err.data_ptr()) if d_err is not None else None,
        ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == capi.OK, lib.mlbm_last_error(None)


@pytest.mark.gpu
def test_no_alloc_step_matches_handle_step_twice():
    import torch
    from metalbm_gb300 import InputDeck, Lattice, build, capi, fields
    build.build()
    lib = capi.load()
    shape = (24, 20, 16)
    V = int(np.prod(shape))
    amp, lam, axis = 1e-3, 6.0, 1
    deck = InputDeck(latticeT="D3Q19", forcingSchemeT="Guo", forceT="Kolmogorov",
                     relaxationTime=0.6, forceAmplitude=(amp, 0, 0), forceWaveLength=(lam, 1, 1),
                     kolmogorovAxis=axis, globalLength=shape)
    rho, u = fields.perturbed_rest(shape, 3, 0.02, seed=12, rho_amplitude=0.01)

    # the existing entry point: handle, two steps with fused diagnostics
    ref_f, ref_d = [], []
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        f0 = lat.populations()
        for _ in range(2):
            lat.step(1, diagnostics=True)
            ref_f.append(lat.populations())
            ref_d.append(lat.diagnostics())

    # the allocation-free entry point on caller-owned device buffers
    profile = np.array([amp * math.sin(float(i * 2) * math.pi / lam) for i in range(shape[axis])])
    d_f = [_dev(f0, torch), torch.empty(19 * V, dtype=torch.float64, device="cuda"),
           torch.empty(19 * V, dtype=torch.float64, device="cuda")]
    d_prof = _dev(profile, torch)
    d_diag = torch.zeros(5, dtype=torch.float64, device="cuda")
    d_err = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    cfg = deck.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    for k in range(2):
        rc = lib.mlbm_step_f64_noalloc(ct.byref(cfg), ct.c_void_p(d_f[k].data_ptr()),
                                       ct.c_void_p(d_f[k + 1].data_ptr()),
                                       ct.c_void_p(d_prof.data_ptr()),
                                       ct.c_void_p(d_diag.data_ptr()),
                                       ct.c_void_p(d_err.data_ptr()), ct.c_void_p(stream))
        assert rc == capi.OK, lib.mlbm_last_error(None)
        torch.cuda.synchronize()
        got = d_f[k + 1].cpu().numpy().reshape(19, V)
        diag = d_diag.cpu().numpy()
        assert np.array_equal(got, ref_f[k])
        assert diag[0] == ref_d[k]["mass"]
        assert diag[1] / V == ref_d[k]["energy"]
        assert diag[2] == ref_d[k]["max_mach"]
        assert int(d_err.cpu()[0]) == 0


@pytest.mark.gpu
def test_no_alloc_step_rejects_lattices_beyond_its_scratch():
    import torch
    from metalbm_gb300 import InputDeck, capi
    lib = capi.load()
    cfg = InputDeck(latticeT="D3Q19", globalLength=(257, 256, 256)).to_c()
    buf = torch.empty(8, dtype=torch.float64, device="cuda")
    p = ct.c_void_p(buf.data_ptr())
    rc = lib.mlbm_step_f64_noalloc(ct.byref(cfg), p, ct.c_void_p(buf.data_ptr() + 8), None, p,
                                   None, None)
    assert rc == capi.ERR_INVALID
    assert b"allocation-free limit" in lib.mlbm_last_error(None)


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape", [("D2Q13", (20, 16, 1)), ("D3Q33", (12, 10, 8)),
                                           ("D3Q15", (12, 10, 8))])
def test_no_alloc_step_on_the_other_lattices(lattice, shape):
    """D2Q13 / D3Q33 (two-node reach) and D3Q15 with a constant Shan-Chen force:
    the allocation-free step equals the handle step bit for bit."""
    import torch
    from metalbm_gb300 import InputDeck, Lattice, build, capi, fields
    build.build()
    lib = capi.load()
    D = 2 if lattice.startswith("D2") else 3
    V = int(np.prod(shape))
    deck = InputDeck(latticeT=lattice, forcingSchemeT="ShanChen", forceT="Constant",
                     relaxationTime=0.7, forceAmplitude=(2e-4, -1e-4, 1e-4), globalLength=shape)
    rho, u = fields.perturbed_rest(shape, D, 0.02, seed=13, rho_amplitude=0.01)
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        f0 = lat.populations()
        lat.step(1)
        ref = lat.populations()
    Q = f0.shape[0]
    d_in, d_out = _dev(f0, torch), torch.empty(Q * V, dtype=torch.float64, device="cuda")
    d_diag = torch.zeros(5, dtype=torch.float64, device="cuda")
    cfg = deck.to_c()
    rc = lib.mlbm_step_f64_noalloc(ct.byref(cfg), ct.c_void_p(d_in.data_ptr()),
                                   ct.c_void_p(d_out.data_ptr()), None,
                                   ct.c_void_p(d_diag.data_ptr()), None,
                                   ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == capi.OK, lib.mlbm_last_error(None)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy().reshape(Q, V), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,forcing,shape", [
    ("D2Q9", "Guo", (24, 18, 1)), ("D3Q27", "Guo", (12, 10, 8)),
    ("D3Q19", "ExactDifferenceMethod", (10, 12, 9)), ("D2Q9", "ExactDifferenceMethod", (20, 14, 1))])
def test_no_alloc_step_sinusoidal_profiles(lattice, forcing, shape):
    """The Sinusoidal force reads the caller's concatenated per-axis profiles
    (x at 0, y at Lx, z at Lx + Ly; no z table in 2-D): two chained calls equal
    two handle steps bit for bit, populations and diagnostics."""
    import torch
    from metalbm_gb300 import InputDeck, Lattice, build, capi, fields
    build.build()
    lib = capi.load()
    D = 2 if lattice == "D2Q9" else 3
    V = int(np.prod(shape))
    amp, lam = (1e-3, -2e-3, 1.5e-3), (7.0, 5.0, 6.0)
    deck = InputDeck(latticeT=lattice, forcingSchemeT=forcing, forceT="Sinusoidal",
                     relaxationTime=0.65, forceAmplitude=amp, forceWaveLength=lam,
                     globalLength=shape)
    rho, u = fields.perturbed_rest(shape, D, 0.02, seed=14, rho_amplitude=0.01)
    ref_f, ref_d = [], []
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        f0 = lat.populations()
        for _ in range(2):
            lat.step(1, diagnostics=True)
            ref_f.append(lat.populations())
            ref_d.append(lat.diagnostics())
    Q = f0.shape[0]
    d_f = [_dev(f0, torch)] + [torch.empty(Q * V, dtype=torch.float64, device="cuda")
                               for _ in range(2)]
    d_prof = _dev(_sin_profiles(amp, lam, shape, D), torch)
    d_diag = torch.zeros(5, dtype=torch.float64, device="cuda")
    d_err = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    cfg = deck.to_c()
    for k in range(2):
        _call(lib, cfg, d_f[k], d_f[k + 1], d_prof, d_diag, d_err, torch)
        torch.cuda.synchronize()
        assert np.array_equal(d_f[k + 1].cpu().numpy().reshape(Q, V), ref_f[k])
        diag = d_diag.cpu().numpy()
        assert diag[0] == ref_d[k]["mass"] and diag[1] / V == ref_d[k]["energy"]
        assert diag[2] == ref_d[k]["max_mach"]
        assert int(d_err.cpu()[0]) == 0


@pytest.mark.gpu
def test_no_alloc_step_allocates_nothing():
    """After a first call (which loads the library's device code on this
    device), further calls leave the device's free memory unchanged."""
    import torch
    from metalbm_gb300 import InputDeck, build, capi, fields
    from metalbm_gb300.lattice import Lattice
    build.build()
    lib = capi.load()
    shape = (16, 12, 10)
    V = int(np.prod(shape))
    amp, lam = (1e-3, 2e-3, -1e-3), (6.0, 5.0, 4.0)
    deck = InputDeck(latticeT="D3Q19", forcingSchemeT="Guo", forceT="Sinusoidal",
                     relaxationTime=0.6, forceAmplitude=amp, forceWaveLength=lam,
                     globalLength=shape)
    rho, u = fields.perturbed_rest(shape, 3, 0.02, seed=15, rho_amplitude=0.01)
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        f0 = lat.populations()
    a, b = _dev(f0, torch), torch.empty(19 * V, dtype=torch.float64, device="cuda")
    d_prof = _dev(_sin_profiles(amp, lam, shape, 3), torch)
    d_diag = torch.zeros(5, dtype=torch.float64, device="cuda")
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    cfg = deck.to_c()
    _call(lib, cfg, a, b, d_prof, d_diag, d_err, torch)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(6):
        _call(lib, cfg, b if k % 2 else a, a if k % 2 else b, d_prof, d_diag, d_err, torch)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert int(d_err.cpu()[0]) == 0
