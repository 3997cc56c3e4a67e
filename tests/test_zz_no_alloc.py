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
