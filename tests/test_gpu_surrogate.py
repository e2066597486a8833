"""Surrogate: tensor-core training gradients against a float64 CPU oracle,
and a small end-to-end run on ADI-priced options."""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fd_adi_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float64)


def _cpu_grads(net, X, T, M, mimic_rounding):
    """float64 CPU forward/backward of the same network; with mimic_rounding
    the bf16 rounding points of the device pipeline are reproduced."""
    from fd_adi_gb300.surrogate import LAYERS
    P = net.P
    r = _bf if mimic_rounding else (lambda x: x)
    W = [net.Wb[l].cpu().to(torch.float64) for l in range(len(LAYERS))]
    b = [net.b[l].cpu().to(torch.float64) for l in range(len(LAYERS))]
    w = net.loss_weights.cpu().to(torch.float64)
    X = X.cpu().to(torch.float64)
    T = T.cpu().to(torch.float64)
    gW, gb = [], []
    for p in range(P):
        Hs, Ys = [X], []
        H = X
        for l in range(len(LAYERS)):
            Y = H @ W[l][p].T + b[l][p]
            Ys.append(Y)
            if l < len(LAYERS) - 1:
                H = r(torch.nn.functional.silu(Y))
                Hs.append(H)
        dY = torch.zeros_like(Ys[-1])
        dY[:, :2] = 2 * w * (Ys[-1][:, :2] - T) / M
        dY = r(dY)
        gWp, gbp = [None] * len(LAYERS), [None] * len(LAYERS)
        for l in range(len(LAYERS) - 1, -1, -1):
            gWp[l] = dY.T @ Hs[l]
            gbp[l] = dY.sum(0)
            if l > 0:
                s = torch.sigmoid(Ys[l - 1])
                dY = r((dY @ W[l][p]) * (s * (1 + Ys[l - 1] * (1 - s))))
        gW.append(gWp)
        gb.append(gbp)
    return gW, gb


def test_training_gradients_match_cpu_oracle(dev):
    from fd_adi_gb300.surrogate import MLPEnsemble, LAYERS
    M = 256
    net = MLPEnsemble(members=2, seed=3, device=dev)
    g = torch.Generator(device="cpu").manual_seed(1)
    X = torch.zeros(M, 16)
    X[:, :8] = torch.rand(M, 8, generator=g) * 2 - 1
    X = X.to(torch.bfloat16).to(dev)
    T = (torch.randn(M, 2, generator=g)).to(dev)
    net.train_step(X, T, M, lr=0.0)
    net.check()
    bufs = net.bufs(M)
    for mimic, tol in ((True, 2e-3), (False, 5e-2)):
        gW, gb = _cpu_grads(net, X, T, M, mimic)
        for p in range(net.P):
            for l in range(len(LAYERS)):
                got = bufs["dW"][l][p].cpu().to(torch.float64)
                ref = gW[p][l]
                scale = ref.abs().max().item()
                assert (got - ref).abs().max().item() <= tol * scale, (mimic, p, l)
                gotb = bufs["db"][l][p].cpu().to(torch.float64)
                bound = tol * gb[p][l].abs().max().item() + 1e-12
                assert (gotb - gb[p][l]).abs().max().item() <= bound


def test_surrogate_learns_adi_prices_and_gates(dev):
    from fd_adi_gb300.surrogate import Surrogate, adi_price, sobol_queries
    grid = dict(nS=64, nv=32, nt=40)
    Qtr = sobol_queries(4096, seed=1)
    Qte = sobol_queries(512, seed=2)
    t0 = time.perf_counter()
    ptr, dtr = adi_price(Qtr, **grid)
    torch.cuda.synchronize()
    t_adi = (time.perf_counter() - t0) / Qtr.shape[0]
    pte, dte = adi_price(Qte, **grid)
    sur = Surrogate(members=4, seed=0, device=dev)
    # 320 steps: too short for the default's 100-step moment averages, which
    # suit the 6400-step full training; the classic constants fit here
    sur.net.adam = (0.9, 0.999, 1e-8)
    losses = sur.fit(Qtr, ptr, dtr, epochs=40, batch=512, lr=2e-3)
    assert losses[-1] < 0.2 * losses[0]
    Q = torch.as_tensor(Qte, device=dev)
    p, d, spread, fb, cnt = sur.predict(Q)
    p = p.cpu().numpy()
    # the control variate alone (the features' Black-Scholes price)
    _, base, _ = sur.feat(Q)
    p_cv = base[:, 0].cpu().numpy() * Qte[:, 1]
    err_net = np.sqrt(np.mean((p - pte) ** 2))
    err_cv = np.sqrt(np.mean((p_cv - pte) ** 2))
    assert err_net < 0.5 * err_cv, (err_net, err_cv)
    # queries outside the box always fall back to ADI
    Qout = Qte[:128].copy()
    Qout[:, 2] = 4.0                       # T beyond the box
    _, _, _, fbo, _ = sur.predict(torch.as_tensor(Qout, device=dev))
    assert bool(fbo.bool().all())
    # the error gate: an ensemble predicting log10 |error|, calibrated on one
    # half of the held-out draws so that every query there whose price misses
    # the bar (the median error here: this short training is coarse) falls
    # back; on the other half its scores must rank misses above hits
    h = Qte.shape[0] // 2
    e = np.abs(p - pte)
    bar = float(np.median(e[:h]))
    sur.fit_gate(Qtr, ptr, epochs=40, batch=512, lr=2e-3, floor=0.2 * bar)
    tau, frac = sur.calibrate(Qte[:h], pte[:h], bar=bar, margin=0.0)
    _, _, _, fbg, cntg = sur.predict(torch.as_tensor(Qte, device=dev))
    fbg = fbg.cpu().numpy().astype(bool)
    assert int(cntg.item()) == int(fbg.sum())
    assert fbg[:h][e[:h] > bar].all()          # every miss of the calibration half
    assert 0.0 < frac < 1.0
    g = sur.gate_score(torch.as_tensor(Qte[h:], device=dev)).cpu().numpy()
    miss = e[h:] > bar
    assert g[miss].mean() > g[~miss].mean()
    sur.gate_tau = None
    # inference is much cheaper than pricing by ADI
    Qbig = torch.as_tensor(np.tile(Qte, (64, 1)), device=dev)
    sur.predict(Qbig)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sur.predict(Qbig)
    torch.cuda.synchronize()
    t_sur = (time.perf_counter() - t0) / Qbig.shape[0]
    assert t_sur * 100 < t_adi


def test_two_level_surrogate_beats_the_single_level(dev):
    """The coarse-ADI control variate: CoarseADI prices are the batched ADI's
    on the coarse grid; trained on the same 4096 draws, the two-level
    surrogate's held-out error is well below the single-level one's (the
    network only learns the fine - coarse difference, 0.01 RMS here);
    out-of-box queries fall back; the host box test equals the device's."""
    from fd_adi_gb300.surrogate import Surrogate, CoarseADI, adi_price, sobol_queries, in_box
    fine = dict(nS=64, nv=32, nt=40)
    Qtr = sobol_queries(4096, seed=1)
    Qte = sobol_queries(512, seed=2)
    ptr, dtr = adi_price(Qtr, **fine)
    pte, _ = adi_price(Qte, **fine)
    co = CoarseADI(48, 24, 40, chunk=1024)
    ctr, cte = co.price(Qtr), co.price(Qte)
    ref, _ = adi_price(Qte[:100], nS=48, nv=24, nt=40)
    np.testing.assert_allclose(cte[:100], ref, rtol=1e-12, atol=1e-12)
    errs = {}
    for name, coarse in (("one", None), ("two", co)):
        sur = Surrogate(members=4, seed=0, device=dev, coarse=coarse)
        sur.net.adam = (0.9, 0.999, 1e-8)
        sur.fit(Qtr, ptr, dtr, epochs=40, batch=512, lr=2e-3,
                coarse=ctr if coarse is not None else None)
        p = sur.predict(torch.as_tensor(Qte, device=dev),
                        coarse=cte if coarse is not None else None)[0].cpu().numpy()
        errs[name] = float(np.sqrt(np.mean((p - pte) ** 2)))
        if coarse is not None:
            two = sur
    assert errs["two"] < 0.5 * errs["one"], errs
    with pytest.raises(ValueError):
        two.predict(torch.as_tensor(Qte, device=dev))
    # price(): the coarse prices are computed inside; out-of-box queries
    # (T beyond the box) fall back to the fine ADI and get its price
    Qm = Qte[:64].copy()
    Qm[:16, 2] = 4.0
    ib = in_box(Qm)
    assert not ib[:16].any() and ib[16:].all()
    _, _, dev_inbox = two.features(torch.as_tensor(Qm, device=dev), np.ones(64))
    np.testing.assert_array_equal(dev_inbox.cpu().numpy().astype(bool), ib)
    p, _, fbh = two.price(Qm, **fine)
    assert fbh[:16].all()
    pf, _ = adi_price(Qm[:16], **fine)
    np.testing.assert_allclose(p[:16], pf, rtol=1e-12)


@pytest.mark.parametrize("tiles", [200, 33, 1])
def test_fused_inference_matches_layered_forward(dev, tiles):
    """The one-kernel inference against the layer-by-layer tensor-core forward
    on the same bf16 weights: both round activations to bf16 at the same
    points, so they agree to accumulation order (1e-3 of the output scale).
    200 tiles: more tile pairs than SMs, so every CTA loops; 33 and 1: an odd
    tile count leaves each member's last pair with one tile."""
    from fd_adi_gb300.surrogate import MLPEnsemble
    M = 128 * tiles
    net = MLPEnsemble(members=4, seed=5, device=dev)
    g = torch.Generator(device="cpu").manual_seed(2)
    for li in range(len(net.b)):
        net.b[li].copy_(torch.randn(net.b[li].shape, generator=g) * 0.1)
    X = torch.zeros(M, 16)
    X[:, :14] = torch.rand(M, 14, generator=g) * 2 - 1
    X = X.to(torch.bfloat16).to(dev)
    ref = net.forward(X, M, keep_preact=False)[:, :, :2].clone()
    out = net.infer(X, M)
    torch.cuda.synchronize()
    net.check()
    scale = ref.abs().max().item()
    assert scale > 0
    assert (out - ref).abs().max().item() <= 1e-3 * scale
    again = net.infer(X, M)
    torch.cuda.synchronize()
    assert torch.equal(again, out)


def _series(dev, Q, cv=2):
    from fd_adi_gb300.surrogate import Featurizer
    X, base, inbox = Featurizer(dev, cv)(torch.as_tensor(Q, device=dev))
    return base.cpu().numpy()


def _cos(Q):
    from oracle.analytic import heston_cos
    return np.array([float(np.ravel(heston_cos([q[0]], q[1], q[3], q[8], q[2], q[4], q[5], q[6],
                                               q[7], N=2048))[0]) for q in Q])


def test_series_control_variate_error_order_in_sigma(dev):
    """The series control variates (Black-Scholes at the expected mean
    variance plus the expansion in the volatility of variance sigma to order 1
    or 2) leave an O(sigma^2) or O(sigma^3) error against the semi-analytic
    Heston price; the plain Black-Scholes variate leaves O(sigma). A wrong
    first- or second-order coefficient would leave a lower order."""
    sig = np.array([0.02, 0.04, 0.08])
    rows = []
    for K, T, rho in [(80.0, 1.0, -0.7), (90.0, 0.5, -0.4), (115.0, 2.0, -0.9)]:
        for s in sig:
            rows.append([100.0, K, T, 0.03, 2.0, 0.04, s, rho, 0.06])
    Q = np.array(rows)
    ref = _cos(Q) / Q[:, 1]
    e = {cv: np.abs(_series(dev, Q, cv)[:, 0] - ref).reshape(3, 3) for cv in (0, 1, 2)}
    # doubling sigma multiplies the error by 2^order
    for cv, lo, hi in ((0, 1.6, 2.6), (1, 3.0, 5.5), (2, 5.5, 11.0)):
        r = e[cv][:, 1:] / e[cv][:, :-1]
        assert np.all((r > lo) & (r < hi)), (cv, e[cv], r)
    assert np.all(e[1] < 0.15 * e[0]) and np.all(e[2] < 0.05 * e[0])


def test_series_control_variate_across_the_box(dev):
    """Across the training box the order-2 series variate cuts the RMS
    residual against the semi-analytic price by more than 40% (0.705 -> 0.340
    on this sample) and order 1 cuts it too; the delta keeps the
    Black-Scholes variate; the plain variate's residual scales are 1, the
    series' price scale is sigma sqrt(T) + 0.1."""
    from fd_adi_gb300.surrogate import sobol_queries
    Q = sobol_queries(512, seed=7)
    ref = _cos(Q)
    b = {cv: _series(dev, Q, cv) for cv in (0, 1, 2)}
    rms = {cv: np.sqrt(np.mean((b[cv][:, 0] * Q[:, 1] - ref) ** 2)) for cv in b}
    assert rms[2] < 0.6 * rms[0] and rms[1] < rms[0], rms
    np.testing.assert_array_equal(b[0][:, 2:], 1.0)
    for cv in (1, 2):
        np.testing.assert_array_equal(b[cv][:, 1], b[0][:, 1])
        np.testing.assert_allclose(b[cv][:, 2], Q[:, 6] * np.sqrt(Q[:, 2]) + 0.1, rtol=1e-15)
        np.testing.assert_array_equal(b[cv][:, 3], 1.0)


def test_unknown_control_variate_and_bad_queries_are_rejected(dev):
    from fd_adi_gb300.surrogate import Featurizer
    with pytest.raises(ValueError):
        Featurizer(dev, 3)
    f = Featurizer(dev)
    Q = torch.ones(256, 9, dtype=torch.float64, device=dev)
    for bad in (Q.float(), Q.cpu(), Q[:, :8], torch.ones(256, 18, dtype=torch.float64,
                                                          device=dev)[:, ::2]):
        with pytest.raises(ValueError):
            f(bad)
