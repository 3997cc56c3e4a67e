"""Workflows of the drop-in on the GPU: the D2Q9 plain-method configuration
end to end, checkpoint / restart, alpha state, bounded waits."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_d2q9_kolmogorov_1000_steps_matches_oracle_with_diagnostics():
    """The D2Q9 Kolmogorov configuration: D2Q9 BGK FP64, 256^2, tau 0.6, Guo,
    Kolmogorov F_x(y) = 1e-5 sin(2 pi 4 y / 256), rho0 = 1, u ~ U[-1e-4, 1e-4]
    (seed 0), f at equilibrium, 1000 steps; energy, enstrophy and max Mach
    every 100 steps. The GPU state equals the oracle bit for bit at every
    record; the fused energy / Mach reductions agree with the fields."""
    from metalbm_gb300 import InputDeck, Lattice, fields, spectral
    from oracle import OracleConfig, OraclePort
    shape = (256, 256, 1)
    rho, u = fields.perturbed_rest(shape, 2, 1e-4, seed=0)
    deck = InputDeck(latticeT="D2Q9", forcingSchemeT="Guo", forceT="Kolmogorov", relaxationTime=0.6,
                     forceAmplitude=(1e-5, 0, 0), forceWaveLength=(64.0, 1, 1),
                     globalLength=(256, 256, 1))
    port = OraclePort(OracleConfig(lattice="D2Q9", forcing="Guo", force="Kolmogorov", tau=0.6,
                                   amplitude=(1e-5, 0, 0), wavelength=(64.0, 1, 1),
                                   size=(256, 256, 1), threads=8))
    port.init_equilibrium(rho, u)
    records = []
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        for rec in range(10):
            lat.step(100, store=True, diagnostics=True)
            port.step(100)
            fl, d = lat.fields(), lat.diagnostics()
            pf = port.fields()
            assert np.array_equal(lat.populations(), port.populations())
            assert np.array_equal(fl["u"], pf["u"]) and np.array_equal(fl["rho"], pf["rho"])
            e = spectral.energy(pf["rho"], pf["u"])
            assert abs(d["energy"] - e) <= 1e-13 * e
            assert abs(d["max_mach"] - np.sqrt(3 * (pf["u"] ** 2).sum(0)).max()) <= 1e-15
            records.append((100 * (rec + 1), d["energy"], spectral.enstrophy(fl["u"], shape),
                            d["max_mach"]))
    assert all(r[1] > 0 and r[2] > 0 for r in records)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_checkpoint_restart_continues_exactly(storage, tmp_path):
    from metalbm_gb300 import InputDeck, Lattice, fields
    shape = (12, 10, 8)
    rho, u = fields.taylor_green(shape, u0=0.08)
    deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.5005, globalLength=shape,
                     storage=storage, alphaSolver="residual", newtonTolerance=1e-12,
                     deviationThreshold=0.0)
    with Lattice(deck) as a:
        a.init_equilibrium(rho, u)
        a.step(4)
        a.save_checkpoint(tmp_path / "ck.npz")
        a.step(4)
        fa, aa = a.populations(), a.alpha()
    with Lattice.from_checkpoint(tmp_path / "ck.npz") as b:
        b.step(4)
        assert np.array_equal(b.populations(), fa) and np.array_equal(b.alpha(), aa)


@pytest.mark.gpu
def test_alpha_starts_at_two_without_init_equilibrium():
    """create + set_populations: the alpha guesses are 2 (initAlpha), so the
    step equals the init_equilibrium path on the same populations."""
    from metalbm_gb300 import InputDeck, Lattice, fields
    shape = (10, 8, 6)
    rho, u = fields.taylor_green(shape, u0=0.08)
    deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.5005, globalLength=shape)
    with Lattice(deck) as a:
        a.init_equilibrium(rho, u)
        f0 = a.populations()
        a.step(3)
        ref = a.populations()
    with Lattice(deck) as b:
        assert (b.alpha() == 2.0).all()
        b.set_populations(f0)
        b.step(3)
        assert np.array_equal(b.populations(), ref)


@pytest.mark.gpu
def test_sync_gives_up_after_its_timeout():
    """mlbm_sync returns MLBM_ERR_TIMEOUT when the work outlasts the limit,
    leaves the handle usable, and a later unbounded sync succeeds."""
    from metalbm_gb300 import InputDeck, Lattice, MlbmError, capi, fields
    shape = (128, 128, 128)
    rho, u = fields.taylor_green(shape, u0=0.05)
    deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.5005, globalLength=shape,
                     alphaSolver="residual", newtonTolerance=1e-12, deviationThreshold=0.0)
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        lat.step(20)
        with pytest.raises(MlbmError) as e:
            lat.sync(1)
        assert e.value.code == capi.ERR_TIMEOUT
        lat.sync(-1)
        lat.step(1, diagnostics=True)
        assert lat.diagnostics()["solved_nodes"] > 0


@pytest.mark.gpu
def test_cpp_routine_wait_is_bounded(tmp_path):
    """The C++ drop-in's iterate (called with the reference's signature:
    streams and events) bounds its wait for the device: with a zero limit the
    first step's wait gives up with MLBM_ERR_TIMEOUT, reported as exit 6, and
    the process ends cleanly."""
    import subprocess
    from metalbm_gb300 import build, fields
    exe = build.build_routine()
    shape = (128, 128, 128)
    rho, u = fields.taylor_green(shape, u0=0.05)
    np.concatenate([rho.ravel(), u.ravel()]).tofile(tmp_path / "in.bin")
    args = [str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "3", "2", "1", "0",
            "0", repr(0.5005), "0", "0", "0", "1", "1", "1", "128", "128", "128", "0", "1"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 6, (r.returncode, r.stderr)
    assert "not finished after 0 ms" in r.stderr


@pytest.mark.gpu
def test_registered_host_buffers_round_trip():
    """Fields through page-locked, huge-page host arrays equal those through
    ordinary numpy arrays."""
    from metalbm_gb300 import InputDeck, Lattice, fields
    from metalbm_gb300.hostbuf import pinned_array
    import ctypes as ct
    shape = (24, 20, 16)
    V = 24 * 20 * 16
    rho, u = fields.perturbed_rest(shape, 3, 1e-3, seed=4, rho_amplitude=1e-3)
    h_rho, h_u = pinned_array((V,)), pinned_array((3, V))
    h_rho[:] = rho
    h_u[:] = u
    deck = InputDeck(latticeT="D3Q19", relaxationTime=0.6, globalLength=shape, storage="f32")
    with Lattice(deck) as lat:
        lat.init_equilibrium(h_rho, h_u)
        lat.step(3, store=True)
        o_rho, o_u = pinned_array((V,)), pinned_array((3, V))
        dp = ct.POINTER(ct.c_double)
        assert lat._lib.mlbm_get_fields(lat.handle, o_rho.ctypes.data_as(dp),
                                        o_u.ctypes.data_as(dp), None, None, 0) == 0
        ref = lat.fields()
    assert np.array_equal(o_rho, ref["rho"]) and np.array_equal(o_u, ref["u"])


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["f32", "f16_shifted"])
def test_init_in_place_and_rounding(storage):
    """mlbm_init_equilibrium reads page-locked (and, where the device reads
    pageable memory, ordinary) host arrays in place: the same populations as
    from ordinary arrays; the FP32 equilibrium (double-float arithmetic) is
    the FP64 equilibrium of the reference order rounded to float, at most one
    float ulp off in rare near-tie cases; FP16-shifted within one half ulp of
    the scaled deviation."""
    from metalbm_gb300 import InputDeck, Lattice, fields
    from metalbm_gb300.hostbuf import pinned_array
    shape = (24, 20, 16)
    V = 24 * 20 * 16
    rho, u = fields.perturbed_rest(shape, 3, 0.08, seed=5, rho_amplitude=0.05)
    h_rho, h_u = pinned_array((V,)), pinned_array((3, V))
    h_rho[:] = rho
    h_u[:] = u
    out = {}
    for st in ("f64", storage):
        deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.50025,
                         globalLength=shape, storage=st)
        with Lattice(deck) as lat:
            lat.init_equilibrium(h_rho, h_u)
            a = lat.populations()
            lat.init_equilibrium(rho, u)
            b = lat.populations()
        assert np.array_equal(a, b)
        out[st] = a
    f64 = out["f64"]
    if storage == "f32":
        ref = f64.astype(np.float32).astype(np.float64)
        got = out["f32"]
        ulps = np.abs(got - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
        assert ulps.max() <= 1.0
        assert (got == ref).mean() >= 0.9999
    else:
        from oracle import lattice_tables
        _, w = lattice_tables("D3Q27")
        # FP16-shifted storage: h = fp16(fp32((f - w_q) 2^k_q)), k_q =
        # round(log2(1024 / w_q)); the same rounding of the FP64 equilibrium,
        # one FP16 ulp apart in rare near-tie cases
        k = np.select([w > 0.4, w > 0.3, w > 0.1, w > 0.06, w > 0.025, w > 0.01],
                      [11, 12, 13, 14, 15, 16], 18).astype(np.float64)[:, None]
        scale = 2.0 ** k
        h_ref = ((f64 - w[:, None]) * scale).astype(np.float32).astype(np.float16)
        h_got = ((out[storage] - w[:, None]) * scale).astype(np.float16)
        ulp16 = np.spacing(np.abs(h_ref)).astype(np.float64)
        diff = np.abs(h_got.astype(np.float64) - h_ref.astype(np.float64))
        assert (diff <= ulp16).all()
        assert (diff == 0).mean() >= 0.9999


@pytest.mark.gpu
def test_deck_initial_fields_step_like_the_oracle():
    """Lattice.initialize() from the deck's initDensityT = Peak and a
    homogeneous initVelocityVector (Initialize.h:19-116), then BGK steps with
    Guo / Kolmogorov: bit-identical to the oracle from the same fields."""
    from metalbm_gb300 import InputDeck, Lattice
    from metalbm_gb300.fields import reference_initial_fields
    from oracle import OracleConfig, OraclePort
    shape = (16, 12, 10)
    deck = InputDeck(latticeT="D3Q19", forcingSchemeT="Guo", forceT="Kolmogorov",
                     relaxationTime=0.6, forceAmplitude=(1e-4, 0, 0), forceWaveLength=(6.0, 1, 1),
                     globalLength=shape, initDensityT="Peak", initDensityValue=1.0,
                     initVelocityVector=(0.01, -0.005, 0.002))
    with Lattice(deck) as lat:
        lat.initialize()
        lat.step(5)
        f = lat.populations()
    rho, u = reference_initial_fields(shape, 3, "Peak", 1.0, "Homogeneous", (0.01, -0.005, 0.002))
    port = OraclePort(OracleConfig(lattice="D3Q19", forcing="Guo", force="Kolmogorov", tau=0.6,
                                   amplitude=(1e-4, 0, 0), wavelength=(6.0, 1, 1), size=shape))
    port.init_equilibrium(rho, u)
    port.step(5)
    assert np.array_equal(f, port.populations())
