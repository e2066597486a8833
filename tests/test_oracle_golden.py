"""The C oracle against the reference's own outputs (tests/golden/*.npz).

The fixtures were produced by the reference CPU engine (see
tests/golden/make_golden.py). The oracle restates that engine, so its
operators must match bit for bit and its grids to rounding.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import analytic

HV_THETA = 0.5 + np.sqrt(3) / 6


def test_operators_bitwise(golden):
    g = golden("operators")
    r, kappa, theta, sigma, rho = g["params"]
    ops = O.heston_operators(g["S"], g["v"], r, kappa, theta, sigma, rho)
    np.testing.assert_array_equal(ops["A0"], g["A0"])
    np.testing.assert_array_equal(ops["A1"], g["A1"])
    np.testing.assert_array_equal(ops["R0"], g["R0"])
    np.testing.assert_array_equal(ops["R1"], g["R1"])
    np.testing.assert_array_equal(ops["status"], g["status"])
    n0, n1 = g["S"].size, g["v"].size
    M = np.zeros((n0 * n1, n0 * n1))
    for i in range(n0):
        for j in range(n1):
            for a in (-1, 0, 1):
                for b in (-1, 0, 1):
                    ii, jj = i + a, j + b
                    if 0 <= ii < n0 and 0 <= jj < n1:
                        M[i * n1 + j, ii * n1 + jj] += ops["M9"][i * n1 + j, (a + 1) * 3 + (b + 1)]
    np.testing.assert_array_equal(M, g["M"])


SCHED = {
    "douglas": lambda n, dt: [("douglas", n, dt, 0.5)],
    "hv": lambda n, dt: [("hv", n, dt, HV_THETA)],
    "implicit": lambda n, dt: [("implicit", n, dt, 1.0)],
    "smooth": lambda n, dt: [("implicit", 2, dt * 0.5, 1.0), ("hv", n - 1, dt, 0.6)],
    "cs": lambda n, dt: [("cs", n, dt, 0.5)],
    "mcs": lambda n, dt: [("mcs", n, dt, 1.0 / 3)],
}


@pytest.mark.parametrize("case", range(18))
def test_solves_match_reference(golden, case):
    g = golden("solves")
    key = str(g["cases"][case])
    r, kappa, theta, sigma, rho = g["case_params"][case]
    scheme = key.split("_", 1)[1]
    out = O.heston_solve(g["S"], g["v"], r, kappa, theta, sigma, rho, g["V0"],
                         SCHED[scheme](20, 0.01))
    ref = g[key]
    scale = np.abs(ref).max()
    assert np.abs(out - ref).max() <= 1e-12 * scale, key


def test_heston150_full_grid(golden):
    g = golden("heston150")
    S, v = g["S"], g["v"]
    V0 = np.maximum(S[:, None] - 100.0, 0) * np.ones((1, v.size))
    n, dt = 150, 1.0 / 150
    out = O.heston_solve(S, v, 0.06, 1.0, 0.04, 0.2, 0.0, V0,
                         [("implicit", 2, dt * 0.5, 1.0), ("douglas", n - 1, dt, 0.5)])
    idx = tuple(g["idx"])
    # parity tolerances: price 1e-10 relative, grid 1e-9 max-norm
    assert abs(out[idx] - g["price"]) <= 1e-10 * abs(g["price"])
    assert np.abs(out - g["V"]).max() <= 1e-9 * np.abs(g["V"]).max()


def test_heston150_vs_semianalytic(golden):
    g = golden("heston150")
    cos = analytic.heston_cos(100., 100., 0.06, 0.04, 1.0, 1.0, 0.04, 0.2, 0.0)[0, 0]
    # the reference's own accuracy bar (tests/test_HestonOptionGPU.py: rtol 1e-3)
    assert abs(float(g["price"]) - cos) <= 1e-3 * cos


def test_blackscholes(golden):
    g = golden("blackscholes")
    r, var, K = g["params"]
    n, dt = 200, 1.0 / 200
    for name, sched in (("implicit", [("implicit", n, dt, 1.0)]),
                        ("douglas", [("douglas", n, dt, 0.5)]),
                        ("hv", [("hv", n, dt, 0.5)]),
                        ("smooth", [("implicit", 2, dt / 2, 1.0), ("hv", n - 1, dt, 0.6)]),
                        ("cs", [("cs", n, dt, 0.5)]),
                        ("mcs", [("mcs", n, dt, 1.0 / 3)])):
        out = O.bs_solve(g["S"], r, var, g["V0"], sched)
        assert np.abs(out - g[name]).max() <= 1e-11 * np.abs(g[name]).max(), name
    # one-dimensional Craig-Sneyd repeats the Douglas sweep in the reference
    np.testing.assert_array_equal(g["cs"], g["douglas"])
    i = int(np.argmin(np.abs(g["S"] - 100.0)))
    exact = analytic.bs_call(100.0, K, r, var, 1.0)[0]
    assert abs(g["douglas"][i] - exact) <= 1e-3 * exact


BARRIER_SCHED = {
    "implicit": [("implicit", 600, 1.0 / 600, 1.0)],
    "douglas": [("douglas", 150, 1.0 / 150, 0.5)],
    "hv": [("hv", 150, 1.0 / 150, 0.5)],
    "smooth": [("implicit", 4, 1.0 / 300, 1.0), ("hv", 148, 1.0 / 150, 0.6)],
}


@pytest.mark.parametrize("scheme", sorted(BARRIER_SCHED))
def test_barrier_vs_reference(golden, scheme):
    """Up-and-out call of the reference's barrier test (rho = 0.4, theta =
    0.12, barrier 170, 150 x 80): the oracle with the barrier's Dirichlet-0
    spot boundary against the reference engine's grids."""
    g = golden("barrier")
    ref = g[scheme]
    got = O.heston_solve(g["S"], g["v"], *g["params"], g["V0"], BARRIER_SCHED[scheme],
                         barrier=True)
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()
    i, j = g["idx"]
    assert abs(got[i, j] - ref[i, j]) <= 1e-13 * abs(ref[i, j])
    # the barrier row stays at the Dirichlet value
    assert np.abs(got[-1]).max() <= 1e-12 * np.abs(got).max()


def test_oracle_constant_rates_match_constant_run():
    """The oracle's per-step rebuild with every step at the option's own r is
    the constant-coefficient solve, bit for bit; a rising rate changes it."""
    from fd_adi_gb300 import mesh
    S, v = mesh.heston_meshes(100., 95., 0.05, 40, 20, 760., 5.)
    V0 = np.maximum(S[:, None] - 95., 0) * np.ones((1, v.size))
    sch = [("implicit", 2, 0.025, 1.0), ("hv", 9, 0.05, HV_THETA)]
    p = (0.03, 2.0, 0.05, 0.6, -0.5)
    a = O.heston_solve(S, v, *p, V0, sch)
    b = O.heston_solve(S, v, *p, V0, sch, rates=np.full(11, 0.03))
    np.testing.assert_array_equal(a, b)
    c = O.heston_solve(S, v, *p, V0, sch, rates=np.linspace(0.01, 0.06, 11))
    assert np.abs(c - a).max() > 1e-3
    with pytest.raises(ValueError):
        O.heston_solve(S, v, *p, V0, sch, rates=np.full(10, 0.03))


UPWIND_SCHED = {
    "douglas": [("douglas", 20, 0.01, 0.5)],
    "hv": [("hv", 20, 0.01, HV_THETA)],
    "implicit": [("implicit", 20, 0.01, 1.0)],
    "smooth": [("implicit", 2, 0.005, 1.0), ("hv", 19, 0.01, 0.6)],
    "cs": [("cs", 20, 0.01, 0.5)],
    "mcs": [("mcs", 20, 0.01, 1.0 / 3)],
}


@pytest.mark.parametrize("tag", ["s", "v", "sv"])
@pytest.mark.parametrize("scheme", sorted(UPWIND_SCHED))
def test_upwind_schemes_vs_reference(golden, tag, scheme):
    """Switched first-derivative schemes (forward in S from the strike's
    index, backward in v from the mean variance's) against the reference
    engine: HV, Douglas and smooth on the diagonalized operators (whose inner
    +-2 entries the reference drops), implicit and Craig-Sneyd on the full
    band."""
    g = golden("upwind")
    fs, fv = (int(x) for x in g["flips"])
    flips = {"s": (fs, None), "v": (None, fv), "sv": (fs, fv)}[tag]
    got = O.heston_solve(g["S"], g["v"], *g["params"], g["V0"], UPWIND_SCHED[scheme],
                         flip_spot=flips[0], flip_var=flips[1])
    ref = g["%s_%s" % (tag, scheme)]
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
