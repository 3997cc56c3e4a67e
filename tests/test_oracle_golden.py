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


CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


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


@pytest.mark.parametrize("lattice", ["D2Q9", "D3Q19", "D3Q27"])
def test_lattice_isotropy(lattice):
    """Known answers of TestLattice.cpp (re-derived): sum w = 1, sum w c = 0,
    sum w c c = cs2 delta, third moment 0, fourth = cs2^2 (dd + dd + dd)."""
    c, w = lattice_tables(lattice)
    D = 2 if lattice == "D2Q9" else 3
    c = c[:, :D]
    cs2 = 1.0 / 3.0
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.abs(np.einsum("q,qa->a", w, c)).max() < 1e-15
    assert np.abs(np.einsum("q,qa,qb->ab", w, c, c) - cs2 * np.eye(D)).max() < 1e-15
    assert np.abs(np.einsum("q,qa,qb,qc->abc", w, c, c, c)).max() < 1e-15
    I = np.eye(D)
    iso4 = cs2 ** 2 * (np.einsum("ab,cd->abcd", I, I) + np.einsum("ac,bd->abcd", I, I)
                       + np.einsum("ad,bc->abcd", I, I))
    assert np.abs(np.einsum("q,qa,qb,qc,qd->abcd", w, c, c, c, c) - iso4).max() < 1e-15
    # opposite velocities: faceQ populations with c_x=-1 then their +1 mirrors
    assert (c[0] == 0).all()


@pytest.mark.parametrize("lattice", ["D2Q9", "D3Q19", "D3Q27"])
def test_equilibrium_moments(lattice):
    """TestMoment.cpp:68-95 idea: moments of f_eq(rho,u) give back rho and rho u."""
    c, w = lattice_tables(lattice)
    D = 2 if lattice == "D2Q9" else 3
    rho, u = 1.037, np.array([0.011, -0.02, 0.007])[:D]
    feq = np.array([equilibrium(lattice, rho, u, q) for q in range(len(w))])
    assert abs(feq.sum() - rho) < 1e-14
    assert np.abs(feq @ c[:, :D] - rho * u).max() < 1e-14


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
