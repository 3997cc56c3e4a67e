"""The FP32-storage entropic kernel's entropy function against an
extended-precision evaluation of its definition (EntropicStep.h:31-62).

F(x) = sum f ln(f/w) - sum g ln(g/w), g = f - x f_neq, and
F'(x) = sum f_neq (1 + ln(g/w)), evaluated in numpy's long double on the host.
The kernel evaluates F in the moment-series form for max|f_neq/f| <= 0.0125
and in the log1p form otherwise. The series form carries a per-node error
bound that the solve subtracts from the residual tolerance (1e-12); the test
checks that bound (and a fixed 4e-15 for the log1p form) against the
definition.
"""
import ctypes as ct

import numpy as np
import pytest

from oracle.port import lattice_tables

LATTICES = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}
F_BOUND = 4e-15  # absolute, 0.4% of the residual tolerance 1e-12 (log1p form)


def series_bound(rmax, rho):
    """The series form's evaluation-error bound for FP32 storage (the kernel's
    series_error_bound): FP32 M3 below rmax = 2.5e-3, FP32 M5 above, B1 and
    M2 in double-float arithmetic, FP64 rounding."""
    m = np.where(rmax <= 0.0025, 6.0e-6 * rmax ** 3, 1.2e-5 * rmax ** 5)
    return rho * (m + 2.0e-13 * rmax + 3.2e-13 * rmax ** 2) + 1e-15


def make_nodes(lattice, rmax_targets, seed):
    """FP32 populations around a random equilibrium and their exact f_neq."""
    c, w = lattice_tables(lattice)
    Q = w.size
    D = 2 if lattice == "D2Q9" else 3
    rng = np.random.default_rng(seed)
    n = rmax_targets.size
    rho = rng.uniform(0.97, 1.03, n)
    u = np.zeros((n, 3))
    u[:, :D] = rng.uniform(-0.08, 0.08, (n, D))
    cl = c.astype(np.longdouble)
    wl = w.astype(np.longdouble)

    def feq(rho, u):
        cu = u @ cl.T
        u2 = (u * u).sum(1)[:, None]
        P = (3 * cu - 1.5 * u2 + 4.5 * cu * cu - 4.5 * cu * u2 + 4.5 * cu ** 3 + 1.125 * u2 * u2
             - 6.75 * cu * cu * u2 + 3.375 * cu ** 4)
        return rho[:, None] * wl * (1 + P)

    fe = feq(rho.astype(np.longdouble), u.astype(np.longdouble))
    # a deviation pattern with no mass and no momentum, scaled to the target
    dev = rng.standard_normal((n, Q)).astype(np.longdouble) * fe
    basis = np.concatenate([np.ones((1, Q)), c[:, :D].T]).astype(np.longdouble)  # [1+D, Q]
    G = basis @ basis.T
    coef = np.linalg.solve(G.astype(np.float64), (basis @ dev.T).astype(np.float64))
    dev = dev - (coef.T.astype(np.longdouble) @ basis)
    dev *= (rmax_targets[:, None] / np.abs(dev / fe).max(1, keepdims=True))
    f32 = (fe + dev).astype(np.float32)
    fl = f32.astype(np.longdouble)
    rho_f = fl.sum(1)
    u_f = (fl @ cl) / rho_f[:, None]
    fneq = fl - feq(rho_f, u_f)
    return f32, fneq.astype(np.float64), wl


def reference(f32, fneq, wl, xs):
    f = f32.astype(np.longdouble)
    n = fneq.astype(np.longdouble)
    H0 = (f * np.log(f / wl)).sum(1)
    F = np.empty((f.shape[0], xs.size))
    D = np.empty_like(F)
    for i, x in enumerate(xs.astype(np.longdouble)):
        g = f - x * n
        lg = np.log(np.where(g > 0, g, 1) / wl)
        F[:, i] = (H0 - (np.where(g > 0, g * lg, 0)).sum(1)).astype(np.float64)
        D[:, i] = (n * (1 + lg)).sum(1).astype(np.float64)
    return F, D


def evaluate(lattice, f32, fneq, xs, mode):
    from metalbm_gb300 import capi
    lib = capi.load()
    nodes = f32.shape[0]
    F = np.empty((nodes, xs.size))
    D = np.empty_like(F)
    series = np.empty(nodes, dtype=np.int32)
    f32 = np.ascontiguousarray(f32)
    fneq = np.ascontiguousarray(fneq)
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    fp, dp = ct.POINTER(ct.c_float), ct.POINTER(ct.c_double)
    rc = lib.mlbm_testing_entropy(LATTICES[lattice], f32.ctypes.data_as(fp), fneq.ctypes.data_as(dp),
                                  nodes, xs.ctypes.data_as(dp), xs.size, mode, F.ctypes.data_as(dp),
                                  D.ctypes.data_as(dp), series.ctypes.data_as(ct.POINTER(ct.c_int)))
    assert rc == 0
    return F, D, series


@pytest.mark.gpu
@pytest.mark.parametrize("lattice", ["D3Q27", "D3Q19", "D2Q9"])
def test_entropy_forms_match_definition(lattice):
    # targets of max |f_neq / f_eq|; max |f_neq / f| = t / (1 - t) at most
    small = np.geomspace(1e-5, 0.0122, 400)
    large = np.geomspace(0.0135, 0.35, 200)
    f32, fneq, wl = make_nodes(lattice, np.concatenate([small, large]), seed=3)
    xs = np.array([1.0, 1.5, 1.999, 2.0, 2.0005, 2.3, 2.5])
    Fr, Dr = reference(f32, fneq, wl, xs)
    M2 = (fneq ** 2 / f32.astype(np.float64)).sum(1)[:, None]
    F, D, series = evaluate(lattice, f32, fneq, xs, mode=0)
    assert series[:small.size].all() and not series[small.size:].any()
    ok = np.isfinite(Fr)
    f64 = f32.astype(np.float64)
    rmax = np.abs(fneq / f64).max(1)
    bound = np.where(series == 1, series_bound(rmax, f64.sum(1)), F_BOUND)[:, None]
    # the direct form is valid up to alpha_max = min(2.5, 1 / max r_q)
    rpos = (fneq / f64).max(1)
    valid = xs[None, :] <= np.minimum(2.5, 1.0 / np.maximum(rpos, 1e-300))[:, None]
    err = np.abs(F - Fr)
    assert (err <= bound)[valid & ok].all(), (err / bound)[valid & ok].max()
    assert (np.abs(D - Dr)[valid] <= 1e-6 * M2.repeat(xs.size, 1)[valid] + 1e-15).all()
    # both forms on the small-deviation nodes
    Fd, _, sd = evaluate(lattice, f32[:small.size], fneq[:small.size], xs, mode=1)
    Fs, _, ss = evaluate(lattice, f32[:small.size], fneq[:small.size], xs, mode=2)
    assert not sd.any() and ss.all()
    assert np.abs(Fd - Fr[:small.size]).max() <= F_BOUND
    assert (np.abs(Fs - Fr[:small.size]) <= bound[:small.size]).all()
    # the bound stays a small part of the tolerance it is taken from
    assert series_bound(0.0125, 1.03) < 0.1e-12 and series_bound(0.0025, 1.03) < 0.1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("lattice", ["D3Q27", "D3Q19", "D2Q9"])
def test_neq_double_float_within_bound(lattice):
    """f_neq of the FP32 entropic main pass (exact fixed-point moments, then the
    equilibrium in double-float arithmetic) against a long-double evaluation:
    sum_q |delta f_neq_q| within the 8 2^-48 1.6 rho that its error bound
    assumes, and the FP64 form within FP64 rounding."""
    from metalbm_gb300 import capi
    c, w = lattice_tables(lattice)
    Q = w.size
    rmax = np.geomspace(1e-5, 0.3, 3000)
    f32, fneq_ref, wl = make_nodes(lattice, rmax, seed=7)
    lib = capi.load()
    fp, dp = ct.POINTER(ct.c_float), ct.POINTER(ct.c_double)
    f32 = np.ascontiguousarray(f32)
    out = {}
    for mode in (0, 1):
        n = np.empty((f32.shape[0], Q))
        assert lib.mlbm_testing_neq({"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}[lattice],
                                    f32.ctypes.data_as(fp), f32.shape[0], mode,
                                    n.ctypes.data_as(dp)) == 0
        out[mode] = n
    rho = f32.astype(np.float64).sum(1)
    err_dfl = np.abs(out[1] - fneq_ref).sum(1)
    err_f64 = np.abs(out[0] - fneq_ref).sum(1)
    assert (err_dfl <= 8 * 2.0 ** -48 * 1.6 * rho).all(), (err_dfl / rho).max()
    assert (err_f64 <= 64 * 2.0 ** -53 * rho).all(), (err_f64 / rho).max()
