"""Drive the compat-built reference CPU engine (test infrastructure only).

Imports the modules that ``oracle/build_ref.py`` compiled into
``oracle/_ref/FiniteDifference`` and builds a Heston engine the way the
reference's ``HestonFiniteDifferenceEngine`` does. ``heston.py`` itself cannot
be imported under Python 3 (print statements, numexpr, pylab), so its
coefficient dict (heston.py:302-333), boundary dict (heston.py:335-359) and
grid construction (heston.py:380-406) are restated here in Python 3 and handed
to the reference ``FiniteDifferenceEngineADI`` unchanged. The Black-Scholes
engine's coefficient and boundary dicts (blackscholes.py:197-219) are
restated the same way (``price_bs_option``).

Usable where the reference was compat-built from its sources
(``oracle/build_ref.py``) or where its generated C/C++ was compiled
(``oracle/build_ref.py --from-generated``, the GPU host). Only the tests and
the CPU-baseline leg of ``bench.py`` import this module.
"""
import contextlib
import io
import itertools
import os
import sys

import numpy as np

_REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")


def available():
    """True if the compiled reference modules import on this machine."""
    if not os.path.isdir(os.path.join(_REF, "FiniteDifference")):
        return False
    try:
        _import()
        return True
    except ImportError:
        return False


def _import():
    if _REF not in sys.path:
        sys.path.insert(0, _REF)
    # FiniteDifferenceEngine.pyx:411 calls itertools.izip (Python 2).
    if not hasattr(itertools, "izip"):
        itertools.izip = zip
    import FiniteDifference.FiniteDifferenceEngine as FD  # noqa: E402
    import FiniteDifference.BandedOperator as BO  # noqa: E402
    import FiniteDifference.utils as U  # noqa: E402
    from FiniteDifference.Grid import Grid  # noqa: E402
    return FD, BO, U, Grid


def heston_mesh(S0, K, v0, nS, nv, spot_max, var_max, spotdensity=7.0, varexp=4.0):
    """heston.py:384-406: v = exponential_space(0, v0, var_max, varexp, nv),
    S = sinh_space(K, spot_max, spotdensity, nS); spot pinned to S0."""
    FD, BO, U, Grid = _import()
    with contextlib.redirect_stdout(io.StringIO()):
        vars_ = U.exponential_space(0.0, v0, var_max, varexp, nv, force_exact=True)
        spots = U.sinh_space(K, spot_max, spotdensity, nS, force_exact=True)
    spots = np.array(spots, dtype=float)
    spots[np.argmin(np.abs(spots - S0))] = S0
    return spots, np.array(vars_, dtype=float)


def heston_engine(S0, K, r, v0, kappa, theta, sigma, rho, spots, vars_, barrier=False,
                  flip_spot=None, flip_var=None):
    """A reference FiniteDifferenceEngineADI with the Heston PDE (heston.py:302-359);
    barrier: an up-and-out barrier at the top of the spot mesh, whose spot
    boundaries become Dirichlet 0 at both ends (heston.py:361-370);
    flip_spot / flip_var: spliced 'forward' / 'backward' first-derivative
    schemes from that row on (heston.py:414-439)."""
    FD, BO, U, Grid = _import()

    def mu_s(t, *dim):
        return r * dim[0]

    def gamma2_s(t, *dim):
        return 0.5 * dim[1] * dim[0] ** 2

    def mu_v(t, *dim):
        if np.isscalar(dim[0]):
            if dim[0] == 0:
                return 0
        ret = kappa * (theta - dim[1])
        ret[dim[0] == 0] = 0
        return ret

    def gamma2_v(t, *dim):
        if np.isscalar(dim[0]):
            if dim[0] == 0:
                return 0
        ret = 0.5 * sigma ** 2 * dim[1]
        ret[dim[0] == 0] = 0
        return ret

    def cross(t, *dim):
        return rho * sigma * dim[0] * dim[1]

    coefficients = {(): lambda t: -r, (0,): mu_s, (0, 0): gamma2_s,
                    (1,): mu_v, (1, 1): gamma2_v, (0, 1): cross}
    boundaries = {
        (0,): ((0, lambda t, *dim: 0.0), (1, lambda t, *dim: 1.0)),
        (0, 0): ((0, lambda t, *dim: 0.0), (None, lambda t, *dim: 1.0)),
        (1,): ((None, lambda t, *dim: None), (None, lambda t, *dim: None)),
        (1, 1): ((1, lambda t, *dim: 0), (None, lambda t, *dim: None)),
    }
    if barrier:
        boundaries[(0,)] = (boundaries[(0,)][0], (0, lambda *x: 0.0))
        boundaries[(0, 0)] = boundaries[(0,)]
    schemes = {(0,): [{"scheme": "center"}], (1,): [{"scheme": "center"}]}
    if flip_spot is not None:
        schemes[(0,)].append({"scheme": "forward", "from": int(flip_spot)})
    if flip_var is not None:
        schemes[(1,)].append({"scheme": "backward", "from": int(flip_var)})
    grid = Grid([spots, vars_], initializer=lambda *x: np.maximum(x[0] - K, 0))
    F = FD.FiniteDifferenceEngineADI(grid, coefficients=coefficients,
                                     boundaries=boundaries, schemes=schemes)
    with contextlib.redirect_stdout(io.StringIO()):
        F.init()
    return F


def price_index(spots, vars_, S0, v0):
    """heston.py:461-465: bisect on meshes rounded to 4 decimals."""
    from bisect import bisect_left
    ids = bisect_left(list(np.round(spots, decimals=4)), np.round(S0, decimals=4))
    idv = bisect_left(list(np.round(vars_, decimals=4)), np.round(v0, decimals=4))
    return ids, idv


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def price_option(job):
    """Price one Heston call with the reference engine (for a process pool):
    job = (S0, K, r, kappa, theta, sigma, rho, v0, T, nS, nv, nt[, want_grid]);
    the mesh as the reference builds it (S_max = 8K, v_max = 5), two implicit
    half-steps then HV theta = 1/2 + sqrt(3)/6 for the remaining steps. Returns
    (price, grid-point-steps, seconds of the time loop, final grid or None)."""
    import time
    S0, K, r, kappa, theta, sigma, rho, v0, T, nS, nv, nt = job[:12]
    want_grid = len(job) > 12 and bool(job[12])
    spots, vars_ = heston_mesh(S0, K, v0, int(nS), int(nv), 8.0 * K, 5.0)
    F = heston_engine(S0, K, r, v0, kappa, theta, sigma, rho, spots, vars_)
    V0 = F.grid.domain[-1].copy()
    dt = T / nt
    t0 = time.perf_counter()
    V = quiet(F.solve_implicit, 2, dt * 0.5, initial=V0)
    V = quiet(F.solve_hundsdorferverwer, int(nt) - 1, dt, initial=V,
              theta=0.5 + np.sqrt(3.0) / 6.0)
    t = time.perf_counter() - t0
    return (float(V[price_index(spots, vars_, S0, v0)]), float(nS) * nv * nt, t,
            np.asarray(V) if want_grid else None)


def price_bs_option(job):
    """Price one Black-Scholes call with the reference engine (for a process
    pool): job = (S0, K, r, var, T, nS, nt[, want_grid]); the mesh as
    BlackScholesFiniteDifferenceEngine builds it (blackscholes.py:181-183:
    sinh_space(S0, 1500, 7, nS, force_exact=True)), its operator
    (blackscholes.py:197-219) handed to the reference FiniteDifferenceEngineADI,
    two implicit half-steps then HV theta = 1/2 + sqrt(3)/6. The price is the
    grid value at the mesh point nearest S0 (blackscholes.py:222-228).
    Returns (price, grid-point-steps, seconds of the time loop, grid or None)."""
    import time
    S0, K, r, var, T, nS, nt = job[:7]
    want_grid = len(job) > 7 and bool(job[7])
    FD, BO, U, Grid = _import()
    spots = np.array(quiet(U.sinh_space, S0, 1500.0, 7.0, int(nS), force_exact=True),
                     dtype=float)
    coefficients = {(): lambda t: -r, (0,): lambda t, *d: r * d[0],
                    (0, 0): lambda t, *d: 0.5 * var * d[0] ** 2}
    boundaries = {(0,): ((0, lambda *a: 0.0), (1, lambda t, x: 1.0)),
                  (0, 0): ((0, lambda *a: 0.0), (None, lambda t, x: 1.0))}
    G = Grid([spots], initializer=lambda x: np.maximum(x - K, 0))
    F = FD.FiniteDifferenceEngineADI(G, coefficients=coefficients, boundaries=boundaries,
                                     schemes={})
    quiet(F.init)
    V0 = G.domain[-1].copy()
    dt = T / nt
    t0 = time.perf_counter()
    V = quiet(F.solve_implicit, 2, dt * 0.5, initial=V0)
    V = quiet(F.solve_hundsdorferverwer, int(nt) - 1, dt, initial=V,
              theta=0.5 + np.sqrt(3.0) / 6.0)
    t = time.perf_counter() - t0
    i = int(np.argmin(np.abs(spots - S0)))
    return (float(V[i]), float(nS) * nt, t, np.asarray(V) if want_grid else None)
