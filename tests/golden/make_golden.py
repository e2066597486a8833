"""Generate the golden fixtures in tests/golden/ from the reference engine.

Runs the reference CPU engine (compat-built by ``oracle/build_ref.py`` from the
reference sources) and stores its meshes, operators and solution grids as
compressed ``.npz`` files. The fixtures pin both the C oracle
(``oracle/fdadi_oracle.c``) and the product's host code; the GPU tests compare
the CUDA path against the oracle, which these fixtures pin.

Usage (in a container that has the reference tree):
    python oracle/build_ref.py && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_harness as H  # noqa: E402

HV_THETA = 0.5 + np.sqrt(3) / 6


def dia_rows(op):
    """Reference DIA operator -> row-aligned [5, N] (offsets 2, 1, 0, -1, -2)."""
    N = op.shape[0]
    out = np.zeros((5, N))
    for k, o in enumerate(op.D.offsets):
        o = int(o)
        if abs(o) > 2:
            raise ValueError("offset %d" % o)
        row = 2 - o
        data = op.D.data[k]
        for i in range(N):
            j = i + o
            if 0 <= j < N:
                out[row, i] = data[j]
    return out


def fold_code(s):
    return {"CANNOT_FOLD": 0, "CAN_FOLD": 1, "FOLDED": 2}[s]


def meshes():
    FD, BO, U, Grid = H._import()
    out = {}
    S, v = H.heston_mesh(100., 100., 0.04, 150, 150, 800., 5.)
    out["cfg1_S"], out["cfg1_v"] = S, v
    for K in (80., 100., 120.):
        S, v = H.heston_mesh(100., K, 0.04, 1024, 512, 8 * K, 5.)
        out["cfg2_S_K%d" % K], out["cfg2_v_K%d" % K] = S, v
    S, v = H.heston_mesh(100., 100., 0.04, 150, 150, 1500., 10.)
    out["def_S"], out["def_v"] = S, v
    out["bs_S"] = np.array(H.quiet(U.sinh_space, 100., 5000., 1.0, 150, force_exact=True))
    out["barrier_S"] = np.array(H.quiet(U.exponential_space, 0.0, 100., 170., 1.0 / 3, 60,
                                        force_exact=True))
    for n in (33, 64, 96, 150, 256, 512):
        S, v = H.heston_mesh(100., 93., 0.07, n, max(8, n // 2), 8 * 93., 5.)
        out["var_S_%d" % n], out["var_v_%d" % n] = S, v
    np.savez_compressed(os.path.join(HERE, "meshes.npz"), **out)


def operators():
    out = {}
    S, v = H.heston_mesh(100., 100., 0.04, 10, 8, 800., 5.)
    F = H.heston_engine(100., 100., 0.06, 0.04, 1.3, 0.05, 0.5, -0.7, S, v)
    out["S"], out["v"] = S, v
    out["params"] = np.array([0.06, 1.3, 0.05, 0.5, -0.7])
    out["A0"] = dia_rows(F.operators[0])
    out["R0"] = np.array(F.operators[0].R)
    out["A1"] = dia_rows(F.operators[1])
    out["R1"] = np.array(F.operators[1].R)
    out["M"] = F.operators[(0, 1)].D.toarray()
    out["status"] = np.array([fold_code(F.operators[0].top_fold_status),
                              fold_code(F.operators[0].bottom_fold_status),
                              fold_code(F.operators[1].top_fold_status),
                              fold_code(F.operators[1].bottom_fold_status)])
    # folded v operator: the one HV/Douglas use (1 - theta*dt*A1, diagonalized)
    Li = F.operators[1] * (0.5 * -0.01)
    Li.add(1, inplace=True)
    Li.diagonalize()
    out["Li1_folded"] = dia_rows(Li)
    out["Li1_bottom_factors"] = np.array(Li.bottom_factors)
    rng = np.random.RandomState(7)
    X = rng.rand(S.size, v.size) * 50
    out["X"] = X
    out["apply0"] = F.operators[0].apply(X)
    out["apply1"] = F.operators[1].apply(X)
    out["applyM"] = F.operators[(0, 1)].apply(X)
    Li0 = F.operators[0] * -0.01
    Li0.add(1, inplace=True)
    out["solve0"] = Li0.solve(X)
    out["solve1_folded"] = Li.solve(X)
    np.savez_compressed(os.path.join(HERE, "operators.npz"), **out)


SCHEDULES = {
    "douglas": lambda F, n, dt, V0: (H.quiet(F.solve_douglas, n, dt, initial=V0, theta=0.5),
                                     [("douglas", n, dt, 0.5)]),
    "hv": lambda F, n, dt, V0: (H.quiet(F.solve_hundsdorferverwer, n, dt, initial=V0,
                                        theta=HV_THETA), [("hv", n, dt, HV_THETA)]),
    "implicit": lambda F, n, dt, V0: (H.quiet(F.solve_implicit, n, dt, initial=V0),
                                      [("implicit", n, dt, 1.0)]),
    "smooth": lambda F, n, dt, V0: (H.quiet(F.solve_smooth, n, dt, initial=V0, smoothing_steps=1),
                                    [("implicit", 2, dt * 0.5, 1.0), ("hv", n - 1, dt, 0.6)]),
    "cs": lambda F, n, dt, V0: (H.quiet(F.solve_craigsneyd, n, dt, initial=V0, theta=0.5),
                                [("cs", n, dt, 0.5)]),
    "mcs": lambda F, n, dt, V0: (H.quiet(F.solve_craigsneyd2, n, dt, initial=V0, theta=1.0 / 3),
                                 [("mcs", n, dt, 1.0 / 3)]),
}


def solves():
    out = {}
    S, v = H.heston_mesh(100., 100., 0.04, 24, 16, 800., 5.)
    out["S"], out["v"] = S, v
    cases = []
    for ci, (rho, sigma, kappa, theta) in enumerate(((0.0, 0.2, 1.0, 0.04),
                                                      (-0.7, 0.5, 1.0, 0.04),
                                                      (0.4, 0.3, 1.0, 0.12))):
        F = H.heston_engine(100., 100., 0.06, 0.04, kappa, theta, sigma, rho, S, v)
        V0 = F.grid.domain[-1].copy()
        out["V0"] = V0
        for name, fn in SCHEDULES.items():
            res, sched = fn(F, 20, 0.01, V0)
            key = "c%d_%s" % (ci, name)
            out[key] = res
            cases.append((key, rho, sigma, kappa, theta, name))
    out["cases"] = np.array([c[0] for c in cases])
    out["case_params"] = np.array([[0.06, c[3], c[4], c[2], c[1]] for c in cases])
    np.savez_compressed(os.path.join(HERE, "solves.npz"), **out)


def heston150():
    """150x150, nt=150, two implicit half-steps then Douglas theta=0.5."""
    S, v = H.heston_mesh(100., 100., 0.04, 150, 150, 800., 5.)
    F = H.heston_engine(100., 100., 0.06, 0.04, 1.0, 0.04, 0.2, 0.0, S, v)
    V0 = F.grid.domain[-1].copy()
    n, dt = 150, 1.0 / 150
    V = H.quiet(F.solve_implicit, 2, dt * 0.5, initial=V0)
    V = H.quiet(F.solve_douglas, n - 1, dt, initial=V, theta=0.5)
    idx = H.price_index(S, v, 100., 0.04)
    np.savez_compressed(os.path.join(HERE, "heston150.npz"), S=S, v=v, V=V,
                        price=np.array(V[idx]), idx=np.array(idx))


def heston1024x512_short():
    """The large single grid (1024x512, rho=-0.7, sigma=0.5, K=100, HV theta=1/2+sqrt(3)/6
    after two implicit half-steps), shortened to 3 HV steps of dt=1/1000 so the
    reference finishes in seconds. Stores the price, a down-sampled grid and
    whole-grid checksums."""
    S, v = H.heston_mesh(100., 100., 0.04, 1024, 512, 800., 5.)
    F = H.heston_engine(100., 100., 0.06, 0.04, 1.0, 0.04, 0.5, -0.7, S, v)
    V0 = F.grid.domain[-1].copy()
    dt = 1.0 / 1000
    V = H.quiet(F.solve_implicit, 2, dt * 0.5, initial=V0)
    V = H.quiet(F.solve_hundsdorferverwer, 3, dt, initial=V, theta=HV_THETA)
    idx = H.price_index(S, v, 100., 0.04)
    np.savez_compressed(os.path.join(HERE, "heston1024x512_short.npz"), S=S, v=v,
                        V_sub=V[::16, ::8], price=np.array(V[idx]), idx=np.array(idx),
                        sum=np.array(V.sum()), sumsq=np.array((V * V).sum()),
                        rowsum=V.sum(axis=1), colsum=V.sum(axis=0))


def barrier():
    """Up-and-out call, the reference's barrier test case
    (tests/test_HestonBarrierOptionGPU.py:26-117): S0 = K = 100, r = 0.06,
    v0 = 0.04, T = 1, kappa = 1, theta = 0.12, sigma = 0.3, rho = 0.4, barrier
    170; 150 spots from exponential_space(0, K, 170, 1/3) and 80 variances to
    the engine's default v_max = 10 (heston.py:276-296, 380-400); the high spot
    boundary is Dirichlet 0 (heston.py:361-370). Implicit: 600 steps of 1/600;
    Douglas and HV (theta 0.5): 150 steps of 1/150; smooth: 4 implicit
    half-steps then 148 HV steps at theta 0.6 (solve_smooth's defaults)."""
    FD, BO, U, Grid = H._import()
    K, S0, v0, B = 100., 100., 0.04, 170.
    S = np.array(H.quiet(U.exponential_space, 0.0, K, B, 1.0 / 3, 150, force_exact=True))
    v = np.array(H.quiet(U.exponential_space, 0.0, v0, 10.0, 4.0, 80, force_exact=True))
    S[np.argmin(np.abs(S - S0))] = S0
    params = (0.06, 1.0, 0.12, 0.3, 0.4)
    F = H.heston_engine(S0, K, params[0], v0, params[1], params[2], params[3], params[4], S, v,
                        barrier=True)
    V0 = F.grid.domain[-1].copy()
    out = dict(S=S, v=v, V0=V0, params=np.array(params), barrier=np.array(B))
    out["implicit"] = H.quiet(F.solve_implicit, 600, 1.0 / 600, initial=V0)
    out["douglas"] = H.quiet(F.solve_douglas, 150, 1.0 / 150, initial=V0, theta=0.5)
    out["hv"] = H.quiet(F.solve_hundsdorferverwer, 150, 1.0 / 150, initial=V0, theta=0.5)
    out["smooth"] = H.quiet(F.solve_smooth, 150, 1.0 / 150, initial=V0)
    idx = H.price_index(S, v, S0, v0)
    out["idx"] = np.array(idx)
    np.savez_compressed(os.path.join(HERE, "barrier.npz"), **out)


def heston1024x512_nt1000(cached=None):
    """The large single grid in full: 1024x512, rho=-0.7, sigma=0.5, K=100,
    two implicit half-steps then 999 HV steps (theta=1/2+sqrt(3)/6), dt=1/1000
    (about 4 minutes of the reference engine). Stores the meshes, the price, a
    down-sampled grid and whole-grid checksums. `cached`: an npz with the
    reference's final grid Vr from an earlier run of exactly this."""
    S, v = H.heston_mesh(100., 100., 0.04, 1024, 512, 800., 5.)
    if cached:
        d = np.load(cached)
        assert np.array_equal(d["S"], S) and np.array_equal(d["v"], v)
        V = d["Vr"]
    else:
        F = H.heston_engine(100., 100., 0.06, 0.04, 1.0, 0.04, 0.5, -0.7, S, v)
        V0 = F.grid.domain[-1].copy()
        dt = 1.0 / 1000
        V = H.quiet(F.solve_implicit, 2, dt * 0.5, initial=V0)
        V = H.quiet(F.solve_hundsdorferverwer, 999, dt, initial=V, theta=HV_THETA)
    idx = H.price_index(S, v, 100., 0.04)
    np.savez_compressed(os.path.join(HERE, "heston1024x512_nt1000.npz"), S=S, v=v,
                        V_sub=V[::16, ::8], price=np.array(V[idx]), idx=np.array(idx),
                        sum=np.array(V.sum()), rowsum=V.sum(axis=1), colsum=V.sum(axis=0),
                        vmax=np.array(np.abs(V).max()))


def upwind():
    """Up/down-winding (heston.py:414-439): the spot first derivative switches
    to forward differences from the strike's grid index on (flip_idx_spot),
    the variance first derivative to backward differences from the mean
    variance's (flip_idx_var); 40 x 24 grid, rho = -0.7, sigma = 0.5, both
    switches alone and together, for the implicit, Douglas, HV, smooth,
    Craig-Sneyd and modified Craig-Sneyd solves (20 steps of 0.01)."""
    from bisect import bisect_left
    S, v = H.heston_mesh(100., 100., 0.04, 40, 24, 800., 5.)
    fs = bisect_left(list(np.round(S, decimals=5)), np.round(100., decimals=5))
    fv = bisect_left(list(np.round(v, decimals=5)), np.round(0.04, decimals=5))
    p = (0.06, 1.0, 0.04, 0.5, -0.7)
    out = dict(S=S, v=v, params=np.array(p), flips=np.array([fs, fv]))
    for tag, (a, b) in (("s", (fs, None)), ("v", (None, fv)), ("sv", (fs, fv))):
        F = H.heston_engine(100., 100., p[0], 0.04, p[1], p[2], p[3], p[4], S, v,
                            flip_spot=a, flip_var=b)
        V0 = F.grid.domain[-1].copy()
        out["V0"] = V0
        for name, fn in SCHEDULES.items():
            out["%s_%s" % (tag, name)] = fn(F, 20, 0.01, V0)[0]
    np.savez_compressed(os.path.join(HERE, "upwind.npz"), **out)


def blackscholes():
    """1-D Black-Scholes, the reference test case (tests/test_BlackScholesOption.py:24-75):
    S=100, K=99, r=0.06, var=0.04, T=1, 150 spots to 5000 with density 1."""
    FD, BO, U, Grid = H._import()
    S = np.array(H.quiet(U.sinh_space, 100., 5000., 1.0, 150, force_exact=True))
    r, var, K = 0.06, 0.04, 99.
    coefficients = {(): lambda t: -r, (0,): lambda t, *d: r * d[0],
                    (0, 0): lambda t, *d: 0.5 * var * d[0] ** 2}
    boundaries = {(0,): ((0, lambda *a: 0.0), (1, lambda t, x: 1.0)),
                  (0, 0): ((0, lambda *a: 0.0), (None, lambda t, x: 1.0))}
    G = Grid([S], initializer=lambda x: np.maximum(x - K, 0))
    F = FD.FiniteDifferenceEngineADI(G, coefficients=coefficients, boundaries=boundaries,
                                     schemes={})
    H.quiet(F.init)
    V0 = G.domain[-1].copy()
    out = dict(S=S, V0=V0, params=np.array([r, var, K]))
    out["implicit"] = H.quiet(F.solve_implicit, 200, 1.0 / 200, initial=V0)
    out["douglas"] = H.quiet(F.solve_douglas, 200, 1.0 / 200, initial=V0, theta=0.5)
    out["hv"] = H.quiet(F.solve_hundsdorferverwer, 200, 1.0 / 200, initial=V0, theta=0.5)
    out["smooth"] = H.quiet(F.solve_smooth, 200, 1.0 / 200, initial=V0, smoothing_steps=1)
    # Craig-Sneyd in one dimension: cross_term is 0 without a mixed operator
    # (FiniteDifferenceEngine.pyx:595-613), so the original scheme repeats the
    # Douglas sweep; the modified one adds (1/2 - theta) F(Y2 - V)
    out["cs"] = H.quiet(F.solve_craigsneyd, 200, 1.0 / 200, initial=V0, theta=0.5)
    out["mcs"] = H.quiet(F.solve_craigsneyd2, 200, 1.0 / 200, initial=V0, theta=1.0 / 3)
    np.savez_compressed(os.path.join(HERE, "blackscholes.npz"), **out)


if __name__ == "__main__":
    if not H.available():
        sys.exit("build the reference first: python oracle/build_ref.py")
    meshes()
    operators()
    solves()
    heston150()
    heston1024x512_short()
    blackscholes()
    barrier()
    upwind()
    heston1024x512_nt1000(os.environ.get("FDADI_CFG2_CACHE"))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
