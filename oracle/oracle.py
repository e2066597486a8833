"""ctypes front end of the C oracle (test infrastructure only).

``oracle/fdadi_oracle.c`` restates the reference CPU ADI engine in C. This
module compiles it with gcc (``-ffp-contract=off`` so x86 and Arm hosts give the
same bits) into ``oracle/_build/liboracle.so`` and exposes numpy-level calls.
Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import it; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fdadi_oracle.c")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

SCHEMES = {"implicit": 0, "douglas": 1, "hv": 2, "hundsdorferverwer": 2,
           "cs": 3, "craigsneyd": 3, "mcs": 4, "craigsneyd2": 4}

_lib = None


def build(force=False):
    """Compile the oracle if the shared object is missing or older than its source."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
                               "-ffp-contract=off", "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_int64)
        c_int, c_d = ctypes.c_int, ctypes.c_double
        L.oracle_heston_solve.argtypes = [dp, c_int, dp, c_int, c_d, c_d, c_d, c_d, c_d, c_int,
                                          c_int, ip, ip, dp, dp, dp, dp]
        L.oracle_bs_solve.argtypes = [dp, c_int, c_d, c_d, c_int, ip, ip, dp, dp, dp]
        L.oracle_heston_operators.argtypes = [dp, c_int, dp, c_int, c_d, c_d, c_d, c_d, c_d,
                                              dp, dp, dp, dp, dp, ip]
        L.oracle_heston_batch.argtypes = [c_int, dp, lp, ip, dp, lp, ip, dp, c_int, ip, ip,
                                          dp, dp, dp, lp, c_int, ip, dp]
        for f in (L.oracle_heston_solve, L.oracle_bs_solve, L.oracle_heston_operators,
                  L.oracle_heston_batch):
            f.restype = c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _lp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def _schedule(schedule):
    """schedule: list of (scheme, nsteps, dt, theta)."""
    sc = np.array([SCHEMES[s[0]] for s in schedule], dtype=np.int32)
    ns = np.array([int(s[1]) for s in schedule], dtype=np.int32)
    dt = np.array([float(s[2]) for s in schedule], dtype=np.float64)
    th = np.array([float(s[3]) for s in schedule], dtype=np.float64)
    return sc, ns, dt, th


def _flags(drop_zero_mixed, barrier, flip_spot, flip_var):
    f = int(bool(drop_zero_mixed)) | (2 if barrier else 0)
    if flip_spot is not None:
        f |= (int(flip_spot) + 1) << 8
    if flip_var is not None:
        f |= (int(flip_var) + 1) << 20
    return f


def heston_solve(spots, vars_, r, kappa, theta, sigma, rho, V0, schedule, drop_zero_mixed=False,
                 barrier=False, rates=None, flip_spot=None, flip_var=None):
    """Run a schedule of ADI segments on the reference Heston operators
    (barrier: the top of the spot mesh is an up-and-out barrier; rates: the
    interest rate of every step, the operators rebuilt before each;
    flip_spot / flip_var: the row from which the spot first derivative uses
    forward and the variance first derivative backward differences)."""
    S = np.ascontiguousarray(spots, dtype=np.float64)
    v = np.ascontiguousarray(vars_, dtype=np.float64)
    V = np.array(V0, dtype=np.float64, order="C").copy()
    assert V.shape == (S.size, v.size)
    sc, ns, dt, th = _schedule(schedule)
    rc = lib().oracle_heston_solve(_dp(S), S.size, _dp(v), v.size, r, kappa, theta, sigma, rho,
                                   _flags(drop_zero_mixed, barrier, flip_spot, flip_var),
                                   len(sc), _ip(sc), _ip(ns), _dp(dt),
                                   _dp(th), _dp(V), _rates(rates, int(ns.sum())))
    if rc:
        raise ValueError("oracle_heston_solve failed (%d)" % rc)
    return V


def bs_solve(spots, r, var, V0, schedule):
    S = np.ascontiguousarray(spots, dtype=np.float64)
    V = np.array(V0, dtype=np.float64).copy()
    sc, ns, dt, th = _schedule(schedule)
    rc = lib().oracle_bs_solve(_dp(S), S.size, r, var, len(sc), _ip(sc), _ip(ns), _dp(dt),
                               _dp(th), _dp(V))
    if rc:
        raise ValueError("oracle_bs_solve failed (%d)" % rc)
    return V


def heston_operators(spots, vars_, r, kappa, theta, sigma, rho):
    """Combined operators: dict with A0/A1 [5,N] (offsets 2..-2, row-aligned,
    block-major), R0/R1 [N], M9 [N,9] and fold statuses."""
    S = np.ascontiguousarray(spots, dtype=np.float64)
    v = np.ascontiguousarray(vars_, dtype=np.float64)
    N = S.size * v.size
    A0, A1 = np.zeros((5, N)), np.zeros((5, N))
    R0, R1, M9 = np.zeros(N), np.zeros(N), np.zeros((N, 9))
    st = np.zeros(4, dtype=np.int32)
    rc = lib().oracle_heston_operators(_dp(S), S.size, _dp(v), v.size, r, kappa, theta, sigma,
                                       rho, _dp(A0), _dp(R0), _dp(A1), _dp(R1), _dp(M9), _ip(st))
    if rc:
        raise ValueError("oracle_heston_operators failed (%d)" % rc)
    return dict(A0=A0, R0=R0, A1=A1, R1=R1, M9=M9, status=st)


def _rates(rates, total, n=None):
    if rates is None:
        return None
    r = np.ascontiguousarray(rates, dtype=np.float64)
    want = (total,) if n is None else (n, total)
    if r.shape != want:
        raise ValueError("rates must have shape %s, got %s" % (want, r.shape))
    _rates.keep = r
    return _dp(r)


def heston_batch(meshes, params, V0s, schedule_list, nthreads=None, barriers=None, rates=None):
    """Price a list of options on the CPU, one thread per option.

    meshes: list of (spots, vars); params: [n,5] (r, kappa, theta, sigma, rho);
    V0s: list of initial grids; schedule_list: list (per option) of schedules
    sharing schemes/nsteps/theta but with per-option dt; barriers: per option,
    whether the top of its spot mesh is an up-and-out barrier; rates: [n, total
    steps] per-step interest rates (time-dependent coefficients)."""
    n = len(meshes)
    nS = np.array([m[0].size for m in meshes], dtype=np.int32)
    nv = np.array([m[1].size for m in meshes], dtype=np.int32)
    S = np.concatenate([np.asarray(m[0], np.float64) for m in meshes])
    v = np.concatenate([np.asarray(m[1], np.float64) for m in meshes])
    S_off = np.concatenate([[0], np.cumsum(nS)[:-1]]).astype(np.int64)
    v_off = np.concatenate([[0], np.cumsum(nv)[:-1]]).astype(np.int64)
    sizes = nS.astype(np.int64) * nv
    V_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    V = np.concatenate([np.asarray(x, np.float64).ravel() for x in V0s])
    sc, ns, _, th = _schedule(schedule_list[0])
    dt = np.array([[float(s[2]) for s in sch] for sch in schedule_list], dtype=np.float64)
    P = np.ascontiguousarray(params, dtype=np.float64)
    nthreads = int(nthreads or os.cpu_count() or 1)
    bar = np.zeros(n, dtype=np.int32) if barriers is None else \
        np.ascontiguousarray(barriers, dtype=np.int32)
    rc = lib().oracle_heston_batch(n, _dp(S), _lp(S_off), _ip(nS), _dp(v), _lp(v_off), _ip(nv),
                                   _dp(P), len(sc), _ip(sc), _ip(ns), _dp(dt), _dp(th), _dp(V),
                                   _lp(V_off), nthreads, _ip(bar),
                                   _rates(rates, int(ns.sum()), n))
    if rc:
        raise ValueError("oracle_heston_batch: %d options failed" % rc)
    return [V[V_off[k]:V_off[k] + sizes[k]].reshape(nS[k], nv[k]) for k in range(n)]
