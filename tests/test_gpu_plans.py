"""Every launch plan of the batched engine's line solves against the oracle
and the reference's golden outputs, and the autotuner.

The partitioned spot solve and the pipelined variance solve reassociate the
Thomas recurrences, so they are held to the parity bars (price within
1e-10 relative, grid within 1e-9 of its max-norm), not bit equality.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

HV_THETA = 0.5 + np.sqrt(3) / 6


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fd_adi_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)


@pytest.fixture(scope="module")
def uneven(cuda):
    """Sixteen options, uneven grids (nS 32..96 so some lines are shorter than
    a partitioned plan's segment count), with the oracle's solution.

    Coarse grids with long HV steps can amplify rounding by 1e5: on some seeds
    the oracle built with and without FMA contraction differs by 3e-10 in a
    price, so no reordering of the arithmetic could meet a 1e-10 bar there.
    This seed's batch is well conditioned (that spread is 5e-14 in price and
    9e-13 of the grid's max), so the bars test the plans, not the seed."""
    from fd_adi_gb300 import HestonOption, mesh
    from fd_adi_gb300.batch import payoff_grids
    rng = np.random.RandomState(21)
    opts, meshes = [], []
    for k in range(16):
        K = 100 * rng.uniform(0.7, 1.3)
        v0 = rng.uniform(0.01, 0.16)
        o = HestonOption(spot=100., strike=K, interest_rate=rng.uniform(0, 0.08), variance=v0,
                         tenor=rng.uniform(0.1, 2.0), mean_reversion=rng.uniform(0.5, 5),
                         mean_variance=rng.uniform(0.01, 0.16), vol_of_variance=rng.uniform(0.1, 1),
                         correlation=rng.uniform(-0.9, 0))
        nS = int(rng.choice(np.arange(32, 97, 16)))
        nv = int(rng.choice(np.arange(16, 81, 8)))
        opts.append(o)
        meshes.append(mesh.heston_meshes(100., K, v0, nS, nv, 8 * K, 5.0))
    n = 20
    dts = [o.tenor / n for o in opts]
    V0 = payoff_grids(opts, meshes)
    ref = O.heston_batch(meshes, [o.params() for o in opts], V0,
                         [[("implicit", 2, dt / 2, 1.0), ("hv", n - 1, dt, HV_THETA)] for dt in dts])
    kw = dict(scheme="hv", n_steps=n - 1, dt=dts, theta=HV_THETA, implicit_steps=2,
              implicit_dt_factor=0.5)
    return opts, meshes, V0, ref, kw


def _check(out, opts, meshes, ref):
    from fd_adi_gb300 import mesh as M
    for k in range(len(opts)):
        assert _rel(out[k], ref[k]) < 1e-9, k
        i, j = M.price_index(meshes[k][0], meshes[k][1], 100., opts[k].variance.value)
        assert abs(out[k][i, j] - ref[k][i, j]) <= 1e-10 * abs(ref[k][i, j]), k


@pytest.mark.parametrize("k", range(20), ids=lambda k: "spot%d" % k)
def test_spot_plan_vs_oracle(uneven, k):
    from fd_adi_gb300.batch import HestonBatch, SPOT_PLANS, VAR_PLANS, make_plan
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts, meshes, plan=make_plan(SPOT_PLANS[k], VAR_PLANS[0]), **kw)
    assert b.plan == make_plan(SPOT_PLANS[k], VAR_PLANS[0])
    _check(b.solve(V0), opts, meshes, ref)


@pytest.mark.parametrize("k", range(11), ids=lambda k: "var%d" % k)
def test_var_plan_vs_oracle(uneven, k):
    from fd_adi_gb300.batch import HestonBatch, SPOT_PLANS, VAR_PLANS, make_plan
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts, meshes, plan=make_plan(SPOT_PLANS[0], VAR_PLANS[k]), **kw)
    _check(b.solve(V0), opts, meshes, ref)


@pytest.mark.parametrize("groups,expl", [(2, 0), (3, 0), (4, 0), (1, 2), (2, 2), (4, 3)])
@pytest.mark.parametrize("graph", [False, True])
def test_option_groups_vs_oracle(uneven, groups, expl, graph):
    """Option groups on side streams (direct) or graph branches: each group's
    chain runs in order, explicit stages chained across groups; optionally
    the explicit stage with a few blocks per SM looping over tiles."""
    from fd_adi_gb300.batch import HestonBatch, SPOT_PLANS, VAR_PLANS, make_plan
    opts, meshes, V0, ref, kw = uneven
    plan = make_plan(SPOT_PLANS[0], VAR_PLANS[2], groups, expl)
    b = HestonBatch(opts, meshes, plan=plan, graph=graph, **kw)
    assert b.launches_per_run == groups * (3 * 2 + 6 * 19)
    out = b.solve(V0)
    _check(out, opts, meshes, ref)
    one = HestonBatch(opts, meshes, plan=make_plan(SPOT_PLANS[0], VAR_PLANS[2], 1), **kw)
    for k, x in enumerate(one.solve(V0)):
        np.testing.assert_array_equal(out[k], x)   # same kernels per point: same bits


def test_more_groups_than_options(uneven):
    from fd_adi_gb300.batch import HestonBatch, SPOT_PLANS, VAR_PLANS, make_plan
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts[:3], meshes[:3], plan=make_plan(SPOT_PLANS[0], VAR_PLANS[0], 4),
                    **dict(kw, dt=kw["dt"][:3]))
    assert b.launches_per_run == 3 * (3 * 2 + 6 * 19)
    _check(b.solve(V0[:3]), opts[:3], meshes[:3], ref[:3])


def test_plan_list_is_complete(cuda):
    from fd_adi_gb300.batch import SPOT_PLANS, VAR_PLANS
    assert len(SPOT_PLANS) == 20 and len(VAR_PLANS) == 11


def test_unknown_plan_is_rejected(uneven):
    from fd_adi_gb300.batch import HestonBatch
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts[:2], meshes[:2], **dict(kw, dt=kw["dt"][:2]))
    b.set_plan({"spot_kind": 1, "spot_a": 7, "spot_b": 3, "var_kind": 0, "var_warps": 4})
    with pytest.raises(ValueError, match="plan"):
        b.solve(V0[:2])


@pytest.mark.parametrize("plan", [((1, 32, 32), (1, 4)), ((1, 8, 128), (1, 1)),
                                  ((0, 8, 32), (1, 2))])
def test_heston150_golden_with_plan(cuda, golden, plan):
    """The 150x150 option (2 implicit half-steps + Douglas) against the
    reference's golden output under partitioned and pipelined plans."""
    from fd_adi_gb300.batch import HestonBatch, payoff_grids, make_plan
    from fd_adi_gb300 import HestonOption
    g = golden("heston150")
    opt = HestonOption(spot=100., strike=100., interest_rate=0.06, volatility=0.2, tenor=1.0,
                       mean_reversion=1.0, mean_variance=0.04, vol_of_variance=0.2,
                       correlation=0.0)
    mesh = (g["S"], g["v"])
    n, dt = 150, 1.0 / 150
    b = HestonBatch([opt], [mesh], scheme="douglas", n_steps=n - 1, dt=dt, theta=0.5,
                    implicit_steps=2, implicit_dt_factor=0.5, plan=make_plan(*plan))
    V = b.solve(payoff_grids([opt], [mesh]))[0]
    idx = tuple(g["idx"])
    assert abs(V[idx] - g["price"]) <= 1e-10 * abs(g["price"])
    assert np.abs(V - g["V"]).max() <= 1e-9 * np.abs(g["V"]).max()


@pytest.mark.parametrize("var", [(1, 2), (3, 16), (3, 4)])
def test_heston1024x512_golden_partitioned(cuda, golden, var):
    """1024x512 (long lines: the partitioned solves' case) against the
    reference's golden output."""
    from fd_adi_gb300.batch import HestonBatch, make_plan
    g = golden("heston1024x512_short")
    S, v = g["S"], g["v"]
    V0 = np.maximum(S[:, None] - 100.0, 0) * np.ones((1, v.size))
    b = HestonBatch([(0.06, 1.0, 0.04, 0.5, -0.7)], [(S, v)], scheme="hv", n_steps=3,
                    dt=1.0 / 1000, theta=HV_THETA, implicit_steps=2, implicit_dt_factor=0.5,
                    plan=make_plan((1, 8, 128), var))
    V = b.solve([V0])[0]
    idx = tuple(g["idx"])
    assert abs(V[idx] - g["price"]) <= 1e-10 * abs(g["price"])
    assert np.abs(V[::16, ::8] - g["V_sub"]).max() <= 1e-9 * np.abs(g["V_sub"]).max()
    assert abs(V.sum() - g["sum"]) <= 1e-10 * abs(g["sum"])


def test_tune_keeps_state_and_picks_a_listed_plan(uneven, tmp_path, monkeypatch):
    from fd_adi_gb300 import batch as B
    opts, meshes, V0, ref, kw = uneven
    monkeypatch.setenv("FDADI_TUNE_CACHE", str(tmp_path / "plans.json"))
    b = B.HestonBatch(opts, meshes, **kw)
    V = b.pack(V0)
    before = V.clone()
    plan = b.tune(reps=2, force=True)
    torch.cuda.synchronize()
    assert torch.equal(V, before)       # tuning touches the stage buffers only
    assert (plan["spot_kind"], plan["spot_a"], plan["spot_b"]) in B.SPOT_PLANS
    assert (plan["var_kind"], plan["var_warps"]) in B.VAR_PLANS
    assert 1 <= plan["groups"] <= 4
    b.run(V)
    _check(b.unpack(V), opts, meshes, ref)
    # the plan is cached by shape, in the process and in the JSON file
    assert (tmp_path / "plans.json").exists()
    b2 = B.HestonBatch(opts, meshes, plan="auto", **kw)
    assert b2.plan == plan


def test_tuned_graph_run(uneven):
    """A tuned plan inside the CUDA graph gives the direct run's result."""
    from fd_adi_gb300.batch import HestonBatch
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts, meshes, plan="auto", **kw)
    direct = b.solve(V0)
    gb = HestonBatch(opts, meshes, plan=b.plan, graph=True, **kw)
    out = gb.solve(V0)
    for k in range(len(opts)):
        np.testing.assert_array_equal(out[k], direct[k])


def test_status_flags_failed_options(uneven):
    """Per-option status: a NaN volatility of variance breaks that option's
    variance-line pivots, a NaN step poisons its grid; the other options
    report 0 and keep their oracle results."""
    from fd_adi_gb300 import _lib
    from fd_adi_gb300.batch import HestonBatch
    opts, meshes, V0, ref, kw = uneven
    params = [o.params() for o in opts[:4]]
    params[1] = params[1][:3] + (float("nan"),) + params[1][4:]
    dts = list(kw["dt"][:4])
    dts[2] = float("nan")
    b = HestonBatch(params, meshes[:4], **dict(kw, dt=dts))
    V = b.pack(V0[:4])
    b.run(V)
    st = b.status(V)
    assert st[0] == 0 and st[3] == 0
    assert st[1] & _lib.STATUS_PIVOT
    assert st[2] & _lib.STATUS_NONFINITE
    with pytest.raises(ValueError, match="option 1"):
        b.check(V)
    out = b.unpack(V)
    for k in (0, 3):
        assert _rel(out[k], ref[k]) < 1e-9


def test_greeks_match_host_stencils(uneven):
    """Device delta/gamma at each option's price point against the centred
    non-uniform stencils applied to the returned grid on the host."""
    from fd_adi_gb300 import mesh as M
    from fd_adi_gb300.batch import HestonBatch
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts, meshes, **kw)
    V = b.pack(V0)
    b.run(V)
    idx = b.flat_index()
    p, d, g = (t.cpu().numpy() for t in b.greeks(V, idx))
    out = b.unpack(V)
    for k in range(len(opts)):
        S, v = meshes[k]
        i, j = M.price_index(S, v, 100., opts[k].variance.value)
        di, dn = S[i] - S[i - 1], S[i + 1] - S[i]
        s = di + dn
        w1 = (-dn / (di * s), (-di + dn) / (di * dn), di / (dn * s))
        w2 = (2.0 / (di * s), -2.0 / (di * dn), 2.0 / (dn * s))
        col = out[k][i - 1:i + 2, j]
        assert p[k] == out[k][i, j]
        assert abs(d[k] - np.dot(w1, col)) <= 1e-12 * max(1.0, abs(d[k]))
        assert abs(g[k] - np.dot(w2, col)) <= 1e-10 * max(1.0, abs(g[k]))
        # against the oracle's grid: the parity price bar, delta alike
        cr = ref[k][i - 1:i + 2, j]
        assert abs(d[k] - np.dot(w1, cr)) <= 1e-9 * max(1.0, abs(d[k]))


@pytest.mark.parametrize("scheme,theta", [("cs", 0.5), ("mcs", 1.0 / 3), ("mcs", 0.8)])
def test_craig_sneyd_uneven_batch_vs_oracle(uneven, scheme, theta):
    """Batched Craig-Sneyd / modified Craig-Sneyd after a Rannacher start,
    uneven grids, with option groups, against the oracle."""
    from fd_adi_gb300.batch import HestonBatch, SPOT_PLANS, VAR_PLANS, make_plan
    opts, meshes, V0, ref, kw = uneven
    dts = kw["dt"]
    n = 20
    want = O.heston_batch(meshes, [o.params() for o in opts], V0,
                          [[("implicit", 2, dt / 2, 1.0), (scheme, n - 1, dt, theta)] for dt in dts])
    b = HestonBatch(opts, meshes, **dict(kw, scheme=scheme, theta=theta),
                    plan=make_plan(SPOT_PLANS[0], VAR_PLANS[2], 2))
    _check(b.solve(V0), opts, meshes, want)


@pytest.mark.parametrize("plan", [((0, 1, 128), (0, 4)), ((1, 8, 128), (3, 16)),
                                  ((0, 8, 32), (1, 2)), ((1, 32, 4), (2, 1))])
@pytest.mark.parametrize("scheme", ["hv", "douglas", "mcs"])
def test_minimum_and_ragged_grids_vs_oracle(cuda, plan, scheme):
    """The smallest grids the reference accepts (4 points per line,
    BandedOperator.pyx:43) mixed with ragged ones (sizes that fill no tile,
    chunk or segment evenly) in one batch, against the oracle."""
    from fd_adi_gb300.batch import HestonBatch, make_plan
    sizes = [(4, 4), (5, 7), (17, 33), (4, 40), (33, 4), (6, 5), (64, 37)]
    meshes = [(800.0 * np.linspace(0, 1, a) ** 1.5, 5.0 * np.linspace(0, 1, b) ** 2) for a, b in sizes]
    params = [(0.03 + 0.005 * k, 1.5, 0.05, 0.4, -0.5 + 0.05 * k) for k in range(len(sizes))]
    V0 = [np.maximum(m[0][:, None] - 100.0, 0) * np.ones((1, m[1].size)) for m in meshes]
    theta = {"hv": HV_THETA, "douglas": 0.5, "mcs": 1.0 / 3}[scheme]
    dt, n = 0.01, 10
    b = HestonBatch(params, meshes, scheme=scheme, n_steps=n, dt=dt, theta=theta,
                    implicit_steps=2, implicit_dt_factor=0.5, plan=make_plan(*plan))
    out = b.solve(V0)
    for k, m in enumerate(meshes):
        ref = O.heston_solve(m[0], m[1], *params[k], V0[k],
                             [("implicit", 2, dt / 2, 1.0), (scheme, n, dt, theta)])
        assert np.isfinite(out[k]).all(), sizes[k]
        assert _rel(out[k], ref) < 1e-11, (sizes[k], _rel(out[k], ref))
    assert not b.status(b.pack(out)).any()


@pytest.mark.parametrize("put", [False, True])
def test_device_payoff_matches_host_grid(uneven, put):
    """The payoff built on the device equals the host-built initial grids bit
    for bit."""
    from fd_adi_gb300.batch import HestonBatch
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts, meshes, **kw)
    K = torch.tensor([o.strike for o in opts], dtype=torch.float64, device="cuda")
    V = b.payoff(K, put=put)
    torch.cuda.synchronize()
    for k, (S, v) in enumerate(meshes):
        want = (np.maximum(opts[k].strike - S, 0.0) if put else np.maximum(S - opts[k].strike, 0.0))
        want = want[:, None] * np.ones((1, v.size))
        np.testing.assert_array_equal(b.unpack(V)[k], want)


def test_batch_rejects_bad_arguments(uneven):
    """State, strikes and index tensors are checked before any launch: a wrong
    length, dtype or device raises ValueError instead of reading or writing
    out of bounds."""
    from fd_adi_gb300.batch import HestonBatch
    opts, meshes, V0, ref, kw = uneven
    b = HestonBatch(opts, meshes, **kw)
    K = torch.tensor([o.strike for o in opts], dtype=torch.float64, device="cuda")
    for bad in (K[:-1], K.float(), K.cpu()):
        with pytest.raises(ValueError):
            b.payoff(bad)
    V = b.pack(V0)
    idx = b.flat_index()
    strided = torch.empty(2 * b.total_points, dtype=torch.float64, device="cuda")[::2]
    for badV in (V[:-1], V.float(), V.cpu(), strided):
        for call in (lambda: b.payoff(K, badV), lambda: b.run(badV), lambda: b.status(badV),
                     lambda: b.greeks(badV, idx), lambda: b.gather(badV, idx)):
            with pytest.raises(ValueError):
                call()
    for bad in (idx[:-1], idx.int(), idx.cpu()):
        with pytest.raises(ValueError):
            b.greeks(V, bad)
    for bad in (idx.int(), idx.cpu()):
        with pytest.raises(ValueError):
            b.gather(V, bad)
