"""Batched Black-Scholes on the fused engine (fdadi_bs_*).

Bars: the reference engine's own grids (tests/golden/blackscholes.npz, from
FiniteDifferenceEngine.pyx's solve_* on blackscholes.py's operator) within
1e-11 of the grid's max-norm, as the per-operator path; the oracle on an
uneven batch within 1e-11 of each grid's max-norm and its price within 1e-10
relative; the closed form within the discretisation error.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle import analytic  # noqa: E402

HV_THETA = 0.5 + np.sqrt(3) / 6


@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fd_adi_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


GOLDEN_SCHED = {
    "implicit": lambda n, dt: dict(scheme="douglas", n_steps=0, implicit_steps=n,
                                   implicit_dt_factor=1.0),
    "douglas": lambda n, dt: dict(scheme="douglas", n_steps=n, theta=0.5),
    "hv": lambda n, dt: dict(scheme="hv", n_steps=n, theta=0.5),
    "smooth": lambda n, dt: dict(scheme="hv", n_steps=n - 1, theta=0.6, implicit_steps=2,
                                 implicit_dt_factor=0.5),
    "cs": lambda n, dt: dict(scheme="cs", n_steps=n, theta=0.5),
    "mcs": lambda n, dt: dict(scheme="mcs", n_steps=n, theta=1.0 / 3),
}


@pytest.mark.parametrize("fused", [True, False])
def test_engine_vs_reference_fixture(cuda, golden, fused):
    """BlackScholesFiniteDifferenceEngine, fused (one launch) and per-operator,
    against the reference engine's grids."""
    from fd_adi_gb300 import Option, Grid, BlackScholesFiniteDifferenceEngine
    g = golden("blackscholes")
    r, var, K = g["params"]
    opt = Option(spot=100., strike=K, interest_rate=r, variance=var, tenor=1.0)
    grid = Grid([g["S"]], initializer=lambda x: np.maximum(x - K, 0))
    F = BlackScholesFiniteDifferenceEngine(opt, grid=grid, fused=fused)
    assert F.fused == fused
    n, dt = 200, 1.0 / 200
    for name, fn in (("implicit", lambda: F.solve_implicit(n, dt, initial=g["V0"])),
                     ("douglas", lambda: F.solve_douglas(n, dt, initial=g["V0"], theta=0.5)),
                     ("hv", lambda: F.solve_hundsdorferverwer(n, dt, initial=g["V0"], theta=0.5)),
                     ("smooth", lambda: F.solve_smooth(n, dt, initial=g["V0"],
                                                       smoothing_steps=1))):
        assert _rel(fn(), g[name]) < 1e-11, (name, fused)


def test_batch_of_copies_matches_fixture(cuda, golden):
    """70 copies of the reference case in one batch (three warp groups, the
    last one ragged): every copy equals the fixture under every schedule,
    Craig-Sneyd and modified Craig-Sneyd included."""
    from fd_adi_gb300.batch import BlackScholesBatch
    g = golden("blackscholes")
    r, var, K = g["params"]
    n, dt = 200, 1.0 / 200
    for name, kw in GOLDEN_SCHED.items():
        b = BlackScholesBatch([(r, var)] * 70, [g["S"]] * 70, dt=dt, **kw(n, dt))
        out = b.solve([g["V0"]] * 70)
        for k, x in enumerate(out):
            assert _rel(x, g[name]) < 1e-11, (name, k)
        # identical inputs, identical bits: lanes do not interact
        for x in out[1:]:
            np.testing.assert_array_equal(x, out[0])


def _uneven(n_opt, seed):
    from fd_adi_gb300 import mesh
    rng = np.random.default_rng(seed)
    opts, meshes = [], []
    for _ in range(n_opt):
        K = 100 * rng.uniform(0.7, 1.3)
        r, vol = rng.uniform(0.0, 0.08), rng.uniform(0.1, 0.6)
        nS = int(rng.integers(8, 400)) if rng.random() < 0.9 else int(rng.integers(4, 8))
        S = mesh.sinh_space(100.0, 8 * K, 7.0, nS, force_exact=True)
        opts.append(dict(r=r, var=vol * vol, K=K, T=rng.uniform(0.1, 2.0)))
        meshes.append(np.asarray(S, dtype=np.float64))
    return opts, meshes


@pytest.mark.parametrize("scheme", ["douglas", "hv", "cs", "mcs", "implicit", "smooth"])
def test_uneven_batch_vs_oracle(cuda, scheme):
    """100 options, 4..400 spot points (a few of 4-7 points), r, variance,
    strike and step drawn per option, calls and the oracle's schedule."""
    from fd_adi_gb300.batch import BlackScholesBatch
    opts, meshes = _uneven(100, 11 if scheme != "smooth" else 12)
    nt = 60
    dts = [o["T"] / nt for o in opts]
    if scheme == "implicit":
        kw = dict(scheme="douglas", n_steps=0, implicit_steps=nt, implicit_dt_factor=1.0)
        sched = [[("implicit", nt, dt, 1.0)] for dt in dts]
    elif scheme == "smooth":
        kw = dict(scheme="hv", n_steps=nt - 1, theta=0.6, implicit_steps=2,
                  implicit_dt_factor=0.5)
        sched = [[("implicit", 2, dt / 2, 1.0), ("hv", nt - 1, dt, 0.6)] for dt in dts]
    else:
        th = HV_THETA if scheme == "hv" else 0.5
        kw = dict(scheme=scheme, n_steps=nt, theta=th)
        sched = [[(scheme, nt, dt, th)] for dt in dts]
    b = BlackScholesBatch([(o["r"], o["var"]) for o in opts], meshes, dt=dts, **kw)
    V0 = [np.maximum(S - o["K"], 0.0) for o, S in zip(opts, meshes)]
    got = b.solve(V0)
    # both prefetch depths run the same arithmetic: identical bits
    for pf in (2, 4, 8):
        other = BlackScholesBatch([(o["r"], o["var"]) for o in opts], meshes, dt=dts,
                                  prefetch=pf, **kw).solve(V0)
        for x, y in zip(got, other):
            np.testing.assert_array_equal(x, y)
    for k, (o, S) in enumerate(zip(opts, meshes)):
        ref = O.bs_solve(S, o["r"], o["var"], V0[k], sched[k])
        assert _rel(got[k], ref) <= 1e-11, (scheme, k, S.size, _rel(got[k], ref))
        i = int(np.argmin(np.abs(S - 100.0)))
        if abs(ref[i]) > 1e-8 * np.abs(ref).max():
            assert abs(got[k][i] - ref[i]) <= 1e-10 * abs(ref[i]), (scheme, k)


def test_prices_against_closed_form(cuda):
    """The reference's default meshes (sinh to 1500 clustered at the spot,
    force_exact) at 300 points and 400 HV steps after a Rannacher start:
    within 1e-3 relative of the closed form for calls across strikes (the
    oracle's worst case on these draws is 2.3e-4)."""
    from fd_adi_gb300 import Option
    from fd_adi_gb300.batch import BlackScholesBatch
    rng = np.random.default_rng(5)
    opts = [Option(spot=100., strike=float(K), interest_rate=float(r), variance=float(v) ** 2,
                   tenor=1.0)
            for K, r, v in zip(rng.uniform(80, 120, 64), rng.uniform(0.0, 0.08, 64),
                               rng.uniform(0.15, 0.5, 64))]
    nt = 400
    b, meshes = BlackScholesBatch.from_options(opts, nspots=300, scheme="hv", n_steps=nt - 1,
                                               dt=1.0 / nt, theta=HV_THETA, implicit_steps=2,
                                               implicit_dt_factor=0.5)
    K = torch.tensor([o.strike for o in opts], dtype=torch.float64, device=cuda)
    V = b.payoff(K)
    host = np.concatenate([np.maximum(S - o.strike, 0.0) for o, S in zip(opts, meshes)])
    np.testing.assert_array_equal(V.cpu().numpy(), host)
    b.run(V)
    p = b.gather(V, b.flat_index()).cpu().numpy()
    exact = np.array([analytic.bs_call(100.0, o.strike, o.interest_rate.value,
                                       o.variance.value, 1.0)[0] for o in opts])
    np.testing.assert_allclose(p, exact, rtol=1e-3)
    assert (b.status(V) == 0).all()
    V[b.p_off[3]] = float("nan")
    st = b.status(V)
    assert st[3] == 2 and (np.delete(st, 3) == 0).all()


def test_put_payoff_and_bad_input(cuda):
    from fd_adi_gb300.batch import BlackScholesBatch
    S = np.linspace(0.0, 400.0, 50)
    b = BlackScholesBatch([(0.03, 0.04)] * 3, [S] * 3, scheme="douglas", n_steps=2, dt=0.01)
    K = torch.tensor([90.0, 100.0, 110.0], dtype=torch.float64, device=cuda)
    V = b.payoff(K, put=True)
    np.testing.assert_array_equal(V.cpu().numpy().reshape(3, -1),
                                  np.maximum(np.array([[90.0], [100.0], [110.0]]) - S, 0.0))
    with pytest.raises(ValueError):
        b.run(torch.zeros(10, dtype=torch.float64, device=cuda))
    with pytest.raises(ValueError):
        BlackScholesBatch([(0.03, 0.04)], [S[:3]])
    with pytest.raises(ValueError):
        BlackScholesBatch([(0.03, 0.04)], [S], scheme="nope")
