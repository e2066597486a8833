"""Host parts of the batched Black-Scholes and surrogate paths (no GPU): the
batch's mesh layout against per-option meshes, and the training-box test."""
import numpy as np

from fd_adi_gb300 import mesh
from fd_adi_gb300.batch import bs_meshes_batch
from fd_adi_gb300.surrogate import in_box, BOX_LO, BOX_HI


def test_bs_meshes_batch_matches_per_option_meshes():
    rng = np.random.default_rng(3)
    sizes = rng.choice([4, 7, 64, 96, 300], 200)
    spot = np.where(rng.random(200) < 0.5, 100.0, 87.5)
    out = np.full(int(sizes.sum()), np.nan)
    idx = bs_meshes_batch(spot, sizes, 1500.0, 7.0, True, out=out)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k in range(200):
        S = np.asarray(mesh.sinh_space(spot[k], 1500.0, 7.0, int(sizes[k]), force_exact=True))
        np.testing.assert_array_equal(out[off[k]:off[k + 1]], S)
        assert idx[k] == off[k] + int(np.argmin(np.abs(S - spot[k])))


def _query(f):
    """Queries [n][9] (S0, K, T, r, kappa, theta, sigma, rho, v0) from box
    features (S0/K, T, r, kappa, theta, sigma, rho, v0) with S0 = 100."""
    f = np.atleast_2d(f)
    q = np.empty((f.shape[0], 9))
    q[:, 0] = 100.0
    q[:, 1] = 100.0 / f[:, 0]
    q[:, 2:] = f[:, 1:]
    return q


def test_in_box_edges():
    mid = 0.5 * (BOX_LO + BOX_HI)
    assert in_box(_query(mid)).all()
    for j in range(8):
        for v, want in ((BOX_LO[j], True), (BOX_HI[j], True)):
            f = mid.copy()
            f[j] = v
            # the box test runs on S0/K recomputed from K: allow its rounding
            if j == 0:
                f[j] = v * (1 + 1e-12) if v == BOX_LO[j] else v * (1 - 1e-12)
            assert in_box(_query(f))[0] == want, (j, v)
        span = BOX_HI[j] - BOX_LO[j]
        for v in (BOX_LO[j] - 0.01 * span, BOX_HI[j] + 0.01 * span):
            f = mid.copy()
            f[j] = v
            assert not in_box(_query(f))[0], (j, v)
