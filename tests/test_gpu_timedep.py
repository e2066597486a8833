"""Time-dependent coefficients: a per-step interest rate r_k.

The reference documents preprocess_operators as the per-step rebuild for
time-dependent parameters (FiniteDifferenceEngineGPU.pyx:163-167). Here step k
of a solve (the implicit start first) runs on operators built with r = r_k:
the fused batch rebuilds its operators and line-solve factors before every
step, the per-operator engine rebuilds its combined operators, and the oracle
builds the reference operators afresh for every step. Bars: 1e-11 of the
grid's max-norm against the oracle (the fused kernels agree with it to ~1e-13
on these grids); a constant rate table reproduces the constant-rate run bit
for bit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

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


def _options(n, seed):
    from fd_adi_gb300 import mesh
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        K = 100 * rng.uniform(0.8, 1.2)
        v0 = rng.uniform(0.02, 0.1)
        p = (rng.uniform(0.0, 0.06), rng.uniform(0.5, 3.0), rng.uniform(0.02, 0.1),
             rng.uniform(0.2, 0.8), rng.uniform(-0.8, 0.0))
        nS = int(rng.choice([32, 48, 64, 80]))
        nv = int(rng.choice([16, 24, 32, 40]))
        S, v = mesh.heston_meshes(100.0, K, v0, nS, nv, 8 * K, 5.0)
        V0 = np.maximum(S[:, None] - K, 0.0) * np.ones((1, v.size))
        out.append(dict(p=p, S=S, v=v, V0=V0, T=rng.uniform(0.25, 1.5)))
    return out


def _rates(n, total, seed):
    """A rising term structure per option, different for each option."""
    rng = np.random.default_rng(seed)
    r0 = rng.uniform(0.0, 0.03, n)
    slope = rng.uniform(0.0, 0.05, n)
    return r0[:, None] + slope[:, None] * np.linspace(0.0, 1.0, total)[None, :]


@pytest.mark.parametrize("scheme", ["hv", "douglas"])
def test_fused_rates_vs_oracle(cuda, scheme):
    from fd_adi_gb300.batch import HestonBatch
    opts = _options(6, 31)
    n = 16
    kw = (dict(scheme="hv", n_steps=n - 1, theta=HV_THETA, implicit_steps=2,
               implicit_dt_factor=0.5) if scheme == "hv" else
          dict(scheme="douglas", n_steps=n, theta=0.5))
    total = kw.get("implicit_steps", 0) + kw["n_steps"]
    R = _rates(len(opts), total, 7)
    dts = [o["T"] / n for o in opts]
    for graph in (False, True):
        b = HestonBatch([o["p"] for o in opts], [(o["S"], o["v"]) for o in opts], dt=dts,
                        rates=R, graph=graph, **kw)
        got = b.solve([o["V0"] for o in opts])
        sched = ([[("implicit", 2, dt / 2, 1.0), ("hv", n - 1, dt, HV_THETA)] for dt in dts]
                 if scheme == "hv" else [[("douglas", n, dt, 0.5)] for dt in dts])
        ref = O.heston_batch([(o["S"], o["v"]) for o in opts], [o["p"] for o in opts],
                             [o["V0"] for o in opts], sched, rates=R)
        for k in range(len(opts)):
            assert _rel(got[k], ref[k]) < 1e-11, (graph, k)
    # the rates matter: a constant-r run differs
    flat = HestonBatch([o["p"] for o in opts], [(o["S"], o["v"]) for o in opts], dt=dts,
                       **kw).solve([o["V0"] for o in opts])
    assert max(_rel(a, c) for a, c in zip(got, flat)) > 1e-4


def test_constant_rates_reproduce_constant_run(cuda):
    """A rate table equal to each option's own r gives the constant-rate
    result bit for bit (the per-step rebuild recreates the same operators)."""
    from fd_adi_gb300.batch import HestonBatch
    opts = _options(4, 32)
    kw = dict(scheme="hv", n_steps=9, theta=HV_THETA, implicit_steps=2, implicit_dt_factor=0.5,
              dt=[o["T"] / 10 for o in opts])
    R = np.array([[o["p"][0]] * 11 for o in opts])
    a = HestonBatch([o["p"] for o in opts], [(o["S"], o["v"]) for o in opts], **kw).solve(
        [o["V0"] for o in opts])
    b = HestonBatch([o["p"] for o in opts], [(o["S"], o["v"]) for o in opts], rates=R,
                    **kw).solve([o["V0"] for o in opts])
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("fused", [True, False])
def test_engine_rates_vs_oracle(cuda, fused):
    """HestonFiniteDifferenceEngine with engine.rates set: the fused engine and
    the per-operator path (the reference's per-step call sequence with the
    operators rebuilt every step) against the oracle."""
    from fd_adi_gb300 import Grid, HestonFiniteDifferenceEngine, HestonOption
    o = _options(1, 33)[0]
    r, kappa, theta, sigma, rho = o["p"]
    opt = HestonOption(spot=100., strike=100., interest_rate=r, variance=0.04, tenor=1.0,
                       mean_reversion=kappa, mean_variance=theta, vol_of_variance=sigma,
                       correlation=rho)
    S, v = o["S"], o["v"]
    F = HestonFiniteDifferenceEngine(
        opt, grid=Grid([S.copy(), v.copy()], initializer=lambda *x: np.maximum(x[0] - 100., 0)),
        fused=fused)
    n, dt = 12, 1.0 / 12
    F.rates = _rates(1, n + 1, 8)[0]
    V0 = np.maximum(S[:, None] - 100.0, 0.0) * np.ones((1, v.size))
    got = F.solve_smooth(n, dt, V0, smoothing_steps=1)
    ref = O.heston_solve(S, v, *o["p"], V0, [("implicit", 2, dt / 2, 1.0),
                                              ("hv", n - 1, dt, 0.6)],
                         rates=F.rates[:n + 1], drop_zero_mixed=True)
    assert _rel(got, ref) < 1e-11
    got_hv = F.solve_hundsdorferverwer(n, dt, V0, theta=HV_THETA)
    ref_hv = O.heston_solve(S, v, *o["p"], V0, [("hv", n, dt, HV_THETA)],
                            rates=F.rates[:n], drop_zero_mixed=True)
    assert _rel(got_hv, ref_hv) < 1e-11
    # without rates the engine is back on its constant r
    F.rates = None
    const = F.solve_hundsdorferverwer(n, dt, V0, theta=HV_THETA)
    ref_c = O.heston_solve(S, v, *o["p"], V0, [("hv", n, dt, HV_THETA)], drop_zero_mixed=True)
    assert _rel(const, ref_c) < 1e-11
