"""Parity on the sizes the benchmark prices: the batched workload's grids
(nS 64..512, nv 32..256, nt = 200, HV after a Rannacher start, the tuned
launch plan) and the large single instance (1024 x 512, nt = 1000).

Bars (the parity bar of the fused engine against the reference CPU engine,
FiniteDifferenceEngine.pyx:700-775 for HV and :617-659 for the implicit
start): price within 1e-10 relative, full grid within 1e-9 of the grid's
max-norm. The oracle is the C restatement of that engine; where the
reference engine itself was built on this host, the batched sizes are also
checked against it directly.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

HV_THETA = 0.5 + np.sqrt(3) / 6
PRICE_BAR = 1e-10
GRID_BAR = 1e-9


@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fd_adi_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)


def _draw(rng):
    """One option from the batched workload's parameter box (S0 = 100)."""
    return dict(K=100.0 * rng.uniform(0.7, 1.3), T=rng.uniform(0.1, 2.0),
                r=rng.uniform(0.0, 0.08), kappa=rng.uniform(0.5, 5.0),
                theta=rng.uniform(0.01, 0.16), sigma=rng.uniform(0.1, 1.0),
                rho=rng.uniform(-0.9, 0.0), v0=rng.uniform(0.01, 0.16))


def _price_bar_ok(got, ref):
    return abs(got - ref) <= PRICE_BAR * abs(ref)


def _grid_rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_batched_workload_sizes_vs_oracle(cuda):
    """Nine options, nS in {64, 288, 512} x nv in {32, 144, 256}, nt = 200,
    parameters drawn from the batched workload's box, one tuned batch."""
    from fd_adi_gb300 import mesh
    from fd_adi_gb300.batch import HestonBatch
    rng = np.random.default_rng(20)
    sizes = [(a, b) for a in (64, 288, 512) for b in (32, 144, 256)]
    opts = [_draw(rng) for _ in sizes]
    meshes = [mesh.heston_meshes(100.0, o["K"], o["v0"], nS, nv, 8.0 * o["K"], 5.0)
              for o, (nS, nv) in zip(opts, sizes)]
    params = [(o["r"], o["kappa"], o["theta"], o["sigma"], o["rho"]) for o in opts]
    nt = 200
    dts = [o["T"] / nt for o in opts]
    b = HestonBatch(params, meshes, scheme="hv", n_steps=nt - 1, dt=dts, theta=HV_THETA,
                    implicit_steps=2, implicit_dt_factor=0.5, graph=True, plan="auto")
    V0 = [np.maximum(S[:, None] - o["K"], 0.0) * np.ones((1, v.size))
          for o, (S, v) in zip(opts, meshes)]
    got = b.solve(V0)
    ref = O.heston_batch(meshes, params, V0,
                         [[("implicit", 2, dt / 2, 1.0), ("hv", nt - 1, dt, HV_THETA)]
                          for dt in dts])
    for k, (o, (S, v)) in enumerate(zip(opts, meshes)):
        i, j = mesh.price_index(S, v, 100.0, o["v0"])
        assert _price_bar_ok(got[k][i, j], ref[k][i, j]), (
            sizes[k], got[k][i, j], ref[k][i, j])
        assert _grid_rel(got[k], ref[k]) <= GRID_BAR, (sizes[k], _grid_rel(got[k], ref[k]))

    from oracle import ref_harness as H
    if not H.available():
        return
    # the reference CPU engine itself, one process per option
    import multiprocessing as mp
    jobs = [(100.0, o["K"], o["r"], o["kappa"], o["theta"], o["sigma"], o["rho"], o["v0"],
             o["T"], nS, nv, nt, True) for o, (nS, nv) in zip(opts, sizes)]
    with mp.get_context("spawn").Pool(min(len(jobs), 16)) as pool:
        res = pool.map(H.price_option, jobs, chunksize=1)
    for k, (price, _, _, grid) in enumerate(res):
        S, v = meshes[k]
        i, j = mesh.price_index(S, v, 100.0, opts[k]["v0"])
        assert _price_bar_ok(got[k][i, j], price), (sizes[k], got[k][i, j], price)
        assert _grid_rel(got[k], grid) <= GRID_BAR, (sizes[k], _grid_rel(got[k], grid))


def test_large_single_instance_nt1000_vs_reference(cuda, golden):
    """1024 x 512, nt = 1000 (two implicit half-steps, then 999 HV steps at
    theta = 1/2 + sqrt(3)/6), rho = -0.7, sigma = 0.5, K = 100, tuned plan,
    against the reference engine's own result (price, a down-sampled grid,
    row and column sums) and the oracle's full grid, on the reference's
    meshes."""
    from fd_adi_gb300.batch import HestonBatch
    g = golden("heston1024x512_nt1000")
    S, v = g["S"], g["v"]
    K = 100.0
    p = (0.06, 1.0, 0.04, 0.5, -0.7)
    nt, T = 1000, 1.0
    dt = T / nt
    b = HestonBatch([p], [(S, v)], scheme="hv", n_steps=nt - 1, dt=dt, theta=HV_THETA,
                    implicit_steps=2, implicit_dt_factor=0.5, graph=True, plan="auto")
    V0 = np.maximum(S[:, None] - K, 0.0) * np.ones((1, v.size))
    got = b.solve([V0])[0]
    i, j = g["idx"]
    assert _price_bar_ok(got[i, j], float(g["price"])), (got[i, j], float(g["price"]))
    vmax = float(g["vmax"])
    assert np.abs(got[::16, ::8] - g["V_sub"]).max() <= GRID_BAR * vmax
    # row and column sums of the whole grid: every element within the grid bar
    # bounds a sum of n elements by n times the bar
    n0, n1 = got.shape
    assert np.abs(got.sum(axis=1) - g["rowsum"]).max() <= n1 * GRID_BAR * vmax
    assert np.abs(got.sum(axis=0) - g["colsum"]).max() <= n0 * GRID_BAR * vmax
    ref = O.heston_solve(S, v, *p, V0, [("implicit", 2, dt / 2, 1.0),
                                        ("hv", nt - 1, dt, HV_THETA)])
    assert _price_bar_ok(got[i, j], ref[i, j]), (got[i, j], ref[i, j])
    assert _grid_rel(got, ref) <= GRID_BAR, _grid_rel(got, ref)
