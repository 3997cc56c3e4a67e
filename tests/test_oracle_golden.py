"""Pin the C restatement oracle against vectors produced by the reference.

The golden vectors were generated by running the reference metaLBM CPU path
itself (tests/golden/make_golden.py); the restatement must reproduce them
bit for bit (it keeps the reference's operation order and is built with
-ffp-contract=off).
"""
import json

import numpy as np
import pytest

from oracle import ALPHA_REFERENCE, OracleConfig, OraclePort, lattice_tables
from oracle.port import equilibrium

from conftest import GOLDEN


def load(case):
    z = np.load(GOLDEN / f"{case}.npz")
    return {k: z[k] for k in z.files if k != "meta"}, json.loads(str(z["meta"]))


def port_for(meta, **kw):
    coll = "ELBM" if "ELBM" in meta["collision"] else meta["collision"]
    return OraclePort(OracleConfig(
        lattice=meta["lattice"], collision=coll, forcing=meta["forcing"], force=meta["force"],
        tau=meta["tau"], amplitude=tuple(meta["amp"]), wavelength=tuple(meta["wavelength"]),
        size=tuple(meta["size"]), alpha_mode=ALPHA_REFERENCE, **kw))


CASES_ALL = sorted(p.stem for p in GOLDEN.glob("*.npz"))
# the spectral-force goldens: FFT-based forces, compared within tolerance
SPECTRAL_CASES = [c for c in CASES_ALL
                  if any(k in c for k in ("constantshell", "energyremoval", "turbulent2d"))]
CASES = [c for c in CASES_ALL if c not in SPECTRAL_CASES]


@pytest.mark.parametrize("case", CASES)
def test_port_matches_reference_bit_for_bit(case):
    g, meta = load(case)
    port = port_for(meta)
    port.init_equilibrium(g["rho0"], g["u0"])
    port.step(meta["steps"])
    fl = port.fields()
    assert np.array_equal(port.populations(), g["f"])
    assert np.array_equal(fl["rho"], g["rho"])
    assert np.array_equal(fl["u"], g["u"])
    assert np.array_equal(fl["alpha"], g["alpha"])
    assert np.array_equal(fl["force"], g["force"])


@pytest.mark.parametrize("case", CASES)
def test_port_threads_do_not_change_results(case):
    g, meta = load(case)
    a, b = port_for(meta, threads=1), port_for(meta, threads=3)
    for p in (a, b):
        p.init_equilibrium(g["rho0"], g["u0"])
        p.step(5)
    assert np.array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("variant", ["forcedbnr", "approached", "malaspinas", "essentially1",
                                     "essentially2", "forcednr"])
def test_entropic_variants_equal_elbm_in_reference(variant):
    """The other entropic collision types only redefine calculateAlpha, which
    is not virtual: ELBM::calculateRelaxationTime calls ELBM::calculateAlpha
    (Collision.h:227-241, 351-375), so ForcedBNR, Approached, Malaspinas,
    Essentially1/2 and ForcedNR give ELBM's populations and alpha bit for bit
    (vectors made by the reference built with each type)."""
    a, ma = load("d3q27_elbm_none_none")
    b, mb = load(f"d3q27_{variant}_none_none")
    assert mb["collision"] != "ELBM" and mb["collision"].endswith("_ELBM")
    assert ma["steps"] == mb["steps"] and ma["tau"] == mb["tau"]
    assert np.array_equal(a["rho0"], b["rho0"]) and np.array_equal(a["u0"], b["u0"])
    assert np.array_equal(a["f"], b["f"]) and np.array_equal(a["alpha"], b["alpha"])


# c_s^2 of each lattice and the coefficient of its isotropic fourth moment
# sum w c_a c_b c_c c_d = m4 (dd + dd + dd): m4 = cs2^2 except on D2Q13
LATTICE_MOMENTS = {"D2Q9": (1 / 3, 1 / 9), "D3Q19": (1 / 3, 1 / 9), "D3Q27": (1 / 3, 1 / 9),
                   "D3Q15": (1 / 3, 1 / 9), "D2Q13": (1 / 3, 2 / 15),
                   "D3Q33": (0.4156023517935171, 0.4156023517935171 ** 2)}


@pytest.mark.parametrize("lattice", list(LATTICE_MOMENTS))
def test_lattice_isotropy(lattice):
    """Known answers of TestLattice.cpp (re-derived): sum w = 1, sum w c = 0,
    sum w c c = cs2 delta, third moment 0, fourth isotropic. D2Q13's fourth
    moment is 2/15 (dd + dd + dd), not cs2^2 = 1/9."""
    c, w = lattice_tables(lattice)
    D = 2 if lattice.startswith("D2") else 3
    c = c[:, :D]
    cs2, m4 = LATTICE_MOMENTS[lattice]
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.abs(np.einsum("q,qa->a", w, c)).max() < 1e-15
    assert np.abs(np.einsum("q,qa,qb->ab", w, c, c) - cs2 * np.eye(D)).max() < 1e-15
    assert np.abs(np.einsum("q,qa,qb,qc->abc", w, c, c, c)).max() < 1e-15
    I = np.eye(D)
    iso4 = m4 * (np.einsum("ab,cd->abcd", I, I) + np.einsum("ac,bd->abcd", I, I)
                 + np.einsum("ad,bc->abcd", I, I))
    assert np.abs(np.einsum("q,qa,qb,qc,qd->abcd", w, c, c, c, c) - iso4).max() < 1e-15
    # opposite velocities: faceQ populations with c_x=-1 then their +1 mirrors
    assert (c[0] == 0).all()


@pytest.mark.parametrize("lattice", ["D2Q9", "D3Q19", "D3Q27", "D3Q15", "D3Q33"])
def test_equilibrium_moments(lattice):
    """TestMoment.cpp:68-95 idea: moments of f_eq(rho,u) give back rho and rho u."""
    c, w = lattice_tables(lattice)
    D = 2 if lattice.startswith("D2") else 3
    rho, u = 1.037, np.array([0.011, -0.02, 0.007])[:D]
    feq = np.array([equilibrium(lattice, rho, u, q) for q in range(len(w))])
    assert abs(feq.sum() - rho) < 1e-14
    assert np.abs(feq @ c[:, :D] - rho * u).max() < 1e-14


def test_d2q13_equilibrium_moment_excess():
    """On D2Q13 the TruncationMa3 equilibrium with inv_cs2 = 3
    (Equilibrium.h:14-33) conserves neither mass nor momentum exactly: the
    lattice's fourth moment is 2/15 (dd + dd + dd) instead of cs2^2 = 1/9, so
    sum f_eq = rho (1 + (9/8 - 27/12 + 81/24 * 2/5) |u|^4) = rho (1 + 0.225 |u|^4)
    and sum c f_eq = rho u (1 + (27/6 * 2/5 - 9/2 * 1/3) |u|^2) = rho u (1 + 0.3 |u|^2).
    The reference's D2Q13 runs drift in mass accordingly (goldens d2q13_*)."""
    c, w = lattice_tables("D2Q13")
    rho, u = 1.037, np.array([0.031, -0.02])
    feq = np.array([equilibrium("D2Q13", rho, u, q) for q in range(13)])
    u2 = u @ u
    assert abs((feq.sum() - rho) / (rho * u2 * u2) - 0.225) < 1e-6
    assert np.abs((feq @ c[:, :2] - rho * u) / (rho * u * u2) - 0.3).max() < 1e-6


def test_density_known_answer():
    """TestMoment.cpp:27-45 idea: with f_q = idx + q the pulled density at a node
    of a uniform-in-q field is Q*idx + Q(Q-1)/2 when every pulled node has the
    same idx (a 1-node-thick periodic lattice)."""
    port = OraclePort(OracleConfig(lattice="D2Q9", size=(1, 1, 1)))
    f = (5.0 + np.arange(9.0)).reshape(9, 1)
    port.set_populations(f)
    port.step(1)
    assert port.fields()["rho"][0] == 9 * 5.0 + 9 * 8 / 2


def test_residual_mode_logarithm_accuracy():
    """Tang's table-driven logarithm of the residual solver (oracle copy)
    against libm: within a few ulp of ln 2 absolute, 2 ulp relative away from 1."""
    from oracle.port import fast_log
    rng = np.random.default_rng(1)
    xs = np.concatenate([np.exp(rng.uniform(-700, 700, 5000)), rng.uniform(0.5, 2.0, 5000),
                         [1.0, 2.0, 0.5, 5e-324, 1e-310, 1.7e308]])
    got = np.array([fast_log(x) for x in xs])
    ref = np.log(xs)
    bound = np.maximum(4 * np.spacing(np.log(2.0)), 3 * np.spacing(np.abs(ref)))
    assert (np.abs(got - ref) <= bound).all()
    away = np.abs(ref) >= 0.5
    assert (np.abs(got - ref)[away] <= 2 * np.spacing(np.abs(ref[away]))).all()


def spectral_field(meta, rho0, u0):
    """The restated force field of a spectral golden (oracle/spectral_force.py);
    the reference stores its fields only on the last step, so EnergyRemoval
    reads the initial ones throughout."""
    from oracle import spectral_force as sf
    D = 2 if meta["lattice"].startswith("D2") else 3
    shape = tuple(meta["size"])
    if meta["force"] == "ConstantShell":
        return sf.constant_shell_field(shape, D, meta["amp"], meta["kmin"], meta["kmax"])
    if meta["force"] == "EnergyRemoval":
        return sf.energy_removal_field(rho0, u0, shape, D, meta["amp"], meta["kmin"], meta["kmax"])
    return sf.turbulent_field(rho0, u0, shape, D, meta["amp"], meta["kmin"], meta["kmax"],
                              meta["ramp"], meta["rkmin"], meta["rkmax"])


@pytest.mark.parametrize("case", SPECTRAL_CASES)
def test_spectral_force_restatement_matches_reference(case):
    """2-D ConstantShell / EnergyRemoval / Turbulent2D: the reference, built
    with the DFT stand-in for FFTW (oracle/ref_stub/fftw3-mpi.h), against the
    numpy restatement driving the oracle's force-field mode. FFT and DFT round
    differently: force within 1e-14 max|F|, f within 1e-13, u within 1e-12."""
    g, meta = load(case)
    F = spectral_field(meta, g["rho0"], g["u0"])
    assert np.abs(F - g["force"]).max() <= 1e-14 * np.abs(g["force"]).max()
    port = OraclePort(OracleConfig(lattice=meta["lattice"], collision=meta["collision"],
                                   forcing=meta["forcing"], force="Field", tau=meta["tau"],
                                   size=tuple(meta["size"])))
    port.init_equilibrium(g["rho0"], g["u0"])
    port.set_force_field(F)
    port.step(meta["steps"])
    fl = port.fields()
    assert np.abs(port.populations() - g["f"]).max() <= 1e-13 * np.abs(g["f"]).max()
    assert np.abs(fl["u"] - g["u"]).max() <= 1e-12 * np.abs(g["u"]).max()
    assert np.abs(fl["rho"] - g["rho"]).max() <= 1e-13


def _bisection_golden():
    z = np.load(GOLDEN / "bisection" / "d3q27_nodes.npz")
    return {k: z[k] for k in z.files if k != "meta"}, json.loads(str(z["meta"]))


def residual_bound(g, tol):
    """|alpha - alpha_ref| allowed between a solve that stops at |F| <= tol
    and the reference's, which stops at |step| <= tol: tol / |F'(alpha_ref)|
    plus two step tolerances."""
    _, w = lattice_tables("D3Q27")
    gq = g["f"] - g["alpha"][:, None] * g["fneq"]
    dF = np.sum(g["fneq"] * (1.0 + np.log(gq / w)), axis=1)
    return tol / np.abs(dF) + 2 * tol


def test_oracle_bisection_matches_reference_solver():
    """The oracle's bracketed solver, forced (Newton capped at 0, so every
    node goes through the bisection-Newton update), against the reference's
    own Bisection_NewtonRaphsonSolver with its EntropicStepFunctor
    (EntropicStep.h:15-63, 142-220) on the same node data: every node
    converges in both, to the same root within the two stopping rules."""
    from oracle.port import solve_alpha_nodes
    g, meta = _bisection_golden()
    assert g["converged"].all()
    tol = meta["tolerance"]
    a, flags = solve_alpha_nodes("D3Q27", g["f"], g["fneq"], np.full(len(g["f"]), 2.0), tol,
                                 newton_maxit=0, bisect_maxit=meta["iteration_max"])
    assert (flags == 2).all()  # bracketed solver on every node, no fallback
    assert (np.abs(a - g["alpha"]) <= residual_bound(g, tol)).all()
    # with Newton first (the default caps) the same roots
    a2, flags2 = solve_alpha_nodes("D3Q27", g["f"], g["fneq"], np.full(len(g["f"]), 2.0), tol)
    assert not (flags2 & 4).any()
    assert (np.abs(a2 - g["alpha"]) <= residual_bound(g, tol)).all()
