"""The C-ABI library builds, loads and exports every entry point that
include/mlbm/mlbm.h declares. No GPU compute here: only calls that are valid
without a device (config defaults, error reporting)."""
import ctypes as ct
import re

import pytest

from conftest import ROOT


def header_functions(name="mlbm.h"):
    text = (ROOT / "include" / "mlbm" / name).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mlbm_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from metalbm_gb300 import build, capi
    build.build()
    return capi.load()


def test_header_declares_the_boundary():
    names = header_functions()
    for n in ["mlbm_create", "mlbm_destroy", "mlbm_init_equilibrium", "mlbm_set_populations",
              "mlbm_get_populations", "mlbm_step", "mlbm_get_fields", "mlbm_get_diagnostics",
              "mlbm_set_alpha_model", "mlbm_train_alpha_model", "mlbm_last_error", "mlbm_sync"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    from metalbm_gb300 import capi
    missing = [n for n in header_functions() + header_functions("mlbm_testing.h")
               if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(capi.EXPORTS) == header_functions()
    assert sorted(capi.TESTING_EXPORTS) == header_functions("mlbm_testing.h")


def test_config_defaults_are_the_reference_deck(lib):
    from metalbm_gb300 import capi
    c = capi.Config()
    assert lib.mlbm_config_init(ct.byref(c)) == capi.OK
    assert c.newton_tolerance == 1e-8 and c.newton_max_iterations == 50
    assert c.deviation_threshold == 1e-3 and c.kolmogorov_axis == 1


def test_struct_sizes_match_header(lib):
    """ctypes mirrors of the C structs have the C sizes (checked against a
    tiny C program compiled with the header)."""
    import subprocess, tempfile, pathlib
    from metalbm_gb300 import capi
    src = '#include <stdio.h>\n#include "mlbm/mlbm.h"\nint main(){printf("%zu %zu %zu %zu\\n", sizeof(mlbm_config), sizeof(mlbm_diag), sizeof(mlbm_mlp), sizeof(mlbm_train_cfg));return 0;}\n'
    with tempfile.TemporaryDirectory() as td:
        p = pathlib.Path(td)
        (p / "s.c").write_text(src)
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(p / "s.c"), "-o", str(p / "s")], check=True)
        out = subprocess.run([str(p / "s")], capture_output=True, text=True, check=True).stdout.split()
    assert [int(x) for x in out] == [ct.sizeof(capi.Config), ct.sizeof(capi.Diag),
                                     ct.sizeof(capi.Mlp), ct.sizeof(capi.TrainCfg)]


def test_create_reports_errors_without_aborting(lib):
    from metalbm_gb300 import capi
    c = capi.Config()
    lib.mlbm_config_init(ct.byref(c))
    c.relaxation_time = 0.4  # invalid: tau must exceed 1/2
    h = ct.c_void_p()
    assert lib.mlbm_create(ct.byref(c), ct.byref(h)) == capi.ERR_INVALID
    assert b"relaxation time" in lib.mlbm_last_error(None)
    assert lib.mlbm_create(None, ct.byref(h)) == capi.ERR_INVALID


def test_collision_enum_matches_header_and_deck(lib):
    """Every entropic CollisionType of Options.h:33-36 that the reference can
    run is accepted (they run as ELBM); an out-of-range code is rejected, and
    the deck refuses ForcedNR_ELBM_Forcing with the reason."""
    from metalbm_gb300 import capi
    from metalbm_gb300.lattice import InputDeck
    text = (ROOT / "include" / "mlbm" / "mlbm.h").read_text()
    for name, value in [("BGK", 0), ("ELBM", 1), ("FORCED_BNR_ELBM", 2), ("APPROACHED_ELBM", 3),
                        ("MALASPINAS_ELBM", 4), ("ESSENTIALLY1_ELBM", 5),
                        ("ESSENTIALLY2_ELBM", 6), ("FORCED_NR_ELBM", 7)]:
        assert re.search(rf"\bMLBM_{name} = {value}\b", text), name
        assert getattr(capi, name) == value
    for coll in ["ForcedBNR_ELBM", "Approached_ELBM", "Malaspinas_ELBM", "Essentially1_ELBM",
                 "Essentially2_ELBM", "ForcedNR_ELBM"]:
        assert InputDeck(latticeT="D3Q27", collisionT=coll).to_c().collision >= capi.ELBM
    with pytest.raises(ValueError, match="sweep order"):
        InputDeck(collisionT="ForcedNR_ELBM_Forcing").to_c()
    c = capi.Config()
    lib.mlbm_config_init(ct.byref(c))
    c.collision = 8
    h = ct.c_void_p()
    assert lib.mlbm_create(ct.byref(c), ct.byref(h)) == capi.ERR_INVALID
    assert b"collision" in lib.mlbm_last_error(None)


def test_two_node_lattices_run_with_fp64_storage_only(lib):
    """D2Q13 and D3Q33 (reach two nodes) are FP64-storage lattices: FP32 /
    FP16 storage is refused before any device work, with the reason."""
    from metalbm_gb300 import capi
    for lattice in (capi.D2Q13, capi.D3Q33):
        for storage in (capi.STORAGE_F32, capi.STORAGE_F16_SHIFTED):
            c = capi.Config()
            lib.mlbm_config_init(ct.byref(c))
            c.lattice, c.storage = lattice, storage
            h = ct.c_void_p()
            assert lib.mlbm_create(ct.byref(c), ct.byref(h)) == capi.ERR_INVALID
            assert b"FP64 storage" in lib.mlbm_last_error(None)
    c = capi.Config()
    lib.mlbm_config_init(ct.byref(c))
    c.lattice = 6
    h = ct.c_void_p()
    assert lib.mlbm_create(ct.byref(c), ct.byref(h)) == capi.ERR_INVALID
    assert b"bad lattice" in lib.mlbm_last_error(None)


def test_spectral_force_configurations_are_checked(lib):
    """Spectral forces: shells 0 <= kmin <= kmax with 2 kmax below the
    shortest length; refused before any device work."""
    from metalbm_gb300 import capi
    h = ct.c_void_p()
    cases = [(dict(force_kmax=8), b"spectral shell"),
             (dict(removal_kmax=8), b"spectral shell"),
             (dict(force_kmin=3, force_kmax=2), b"spectral shell")]
    for kw, msg in cases:
        c = capi.Config()
        lib.mlbm_config_init(ct.byref(c))
        c.lattice, c.force = capi.D3Q19, capi.FORCE_TURBULENT_2D
        c.length[0] = c.length[1] = c.length[2] = 16
        for k, v in kw.items():
            setattr(c, k, v)
        assert lib.mlbm_create(ct.byref(c), ct.byref(h)) == capi.ERR_INVALID
        assert msg in lib.mlbm_last_error(None), lib.mlbm_last_error(None)
    c = capi.Config()
    lib.mlbm_config_init(ct.byref(c))
    c.force = 7
    assert lib.mlbm_create(ct.byref(c), ct.byref(h)) == capi.ERR_INVALID
    assert c.removal_kmin == 1 and c.removal_kmax == 2 and c.removal_amplitude[0] == 1e-6


def test_input_deck_from_a_reference_deck():
    """The reference's deck syntax (constexpr definitions, src/Input_prod.in:9-79)
    read into an InputDeck; macro lengths from the caller; unsupported choices
    refused with the reason."""
    from metalbm_gb300.lattice import InputDeck
    deck_text = """
    namespace lbm {
      constexpr LatticeType latticeT = LatticeType::D3Q27;
      constexpr int globalLengthX = GLOBAL_LENGTH_X;  // set by CMake
      constexpr int globalLengthY = GLOBAL_LENGTH_Y;
      constexpr int globalLengthZ = GLOBAL_LENGTH_Z;
      constexpr AlgorithmType algorithmT = AlgorithmType::Pull;
      constexpr dataT relaxationTime = 0.55;
      constexpr CollisionType collisionT = CollisionType::BGK;
      constexpr EquilibriumType equilibriumT = EquilibriumType::TruncationMa3;
      constexpr InitDensityType initDensityT = InitDensityType::Peak;
      constexpr dataT initDensityValue = 1.0;
      constexpr Vector initVelocityVector = { {0.0, 1e-3, 0.0} };
      constexpr ForcingSchemeType forcingSchemeT = ForcingSchemeType::ExactDifferenceMethod;
      constexpr ForceType forceT = ForceType::ConstantShell;
      constexpr Vector forceAmplitude = { {1e1, 1e1, 1e1} };
      constexpr Vector forceWaveLength = { {32.0, 32.0, 32.0} };
      constexpr int forcekMin = 1;
      constexpr int forcekMax = 2;
      constexpr Vector removalForceAmplitude = { {1.e-6, 1.e-6, 1.e-6} };
      constexpr unsigned int writeStep = 2000;
    }
    """
    d = InputDeck.from_reference_deck(deck_text, lengths=(64, 48, 32), storage="f32")
    assert (d.latticeT, d.collisionT, d.forcingSchemeT, d.forceT) == (
        "D3Q27", "BGK", "ExactDifferenceMethod", "ConstantShell")
    assert d.relaxationTime == 0.55 and d.globalLength == (64, 48, 32) and d.storage == "f32"
    assert d.forceAmplitude == (10.0, 10.0, 10.0) and (d.forcekMin, d.forcekMax) == (1, 2)
    assert d.removalForceAmplitude == (1e-6, 1e-6, 1e-6) and d.initDensityT == "Peak"
    assert d.initVelocityVector == (0.0, 1e-3, 0.0)
    d.to_c()  # a valid configuration
    with pytest.raises(ValueError, match="lengths"):
        InputDeck.from_reference_deck(deck_text)
    with pytest.raises(ValueError, match="TruncationMa3"):
        InputDeck.from_reference_deck(deck_text.replace("TruncationMa3", "Incompressible"),
                                      lengths=(8, 8, 8))
    # vectors written with an explicit type name, and a long single-line string
    # that is neither a deck nor a file name: a ValueError, not an OSError
    typed = deck_text.replace("= { {1e1, 1e1, 1e1} }", "= MathVector<dataT, 3>{{1e1, 2e1, -3e1}}")
    d = InputDeck.from_reference_deck(typed, lengths=(8, 8, 8))
    assert d.forceAmplitude == (10.0, 20.0, -30.0)
    with pytest.raises(ValueError):
        InputDeck.from_reference_deck("x" * 5000)
