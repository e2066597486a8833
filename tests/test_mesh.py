"""Host mesh generators against the reference's meshes.

The fixtures were made by the reference's own generators on an x86-64 host.
numpy's sinh and arcsinh differ in the last bit between its x86-64 build
(SIMD library routines) and other hosts, so the reference's meshes do too:
the fixture comparisons are bit for bit on x86-64 and within 1e-14 relative
elsewhere. The batched generators are compared with the per-option ones on
the same host, bit for bit everywhere.
"""
import platform

import numpy as np

from fd_adi_gb300 import mesh as M

FIXTURE_HOST = platform.machine() in ("x86_64", "AMD64")


def _same_as_fixture(a, b):
    if FIXTURE_HOST:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=1e-14, atol=0)


def test_heston_meshes(golden):
    g = golden("meshes")
    S, v = M.heston_meshes(100., 100., 0.04, 150, 150, 800., 5.)
    _same_as_fixture(S, g["cfg1_S"])
    _same_as_fixture(v, g["cfg1_v"])
    S, v = M.heston_meshes(100., 100., 0.04, 150, 150, 1500., 10.)
    _same_as_fixture(S, g["def_S"])
    _same_as_fixture(v, g["def_v"])
    for K in (80, 100, 120):
        S, v = M.heston_meshes(100., float(K), 0.04, 1024, 512, 8.0 * K, 5.)
        _same_as_fixture(S, g["cfg2_S_K%d" % K])
        _same_as_fixture(v, g["cfg2_v_K%d" % K])
    for n in (33, 64, 96, 150, 256, 512):
        S, v = M.heston_meshes(100., 93., 0.07, n, max(8, n // 2), 8 * 93., 5.)
        _same_as_fixture(S, g["var_S_%d" % n])
        _same_as_fixture(v, g["var_v_%d" % n])


def test_bs_and_barrier_meshes(golden):
    g = golden("meshes")
    _same_as_fixture(M.sinh_space(100., 5000., 1.0, 150), g["bs_S"])
    _same_as_fixture(M.barrier_spots(100., 170., 60), g["barrier_S"])


def test_price_index():
    S = np.array([0.0, 50.0, 99.99999, 100.0, 150.0])
    assert M.price_index(S, np.array([0.0, 0.04, 1.0]), 100.0, 0.04) == (2, 1)


def _concat_ref(spot, K, v0, nS, nv, spot_max, var_max):
    ref = [M.heston_meshes(spot, K[k], v0[k], int(nS[k]), int(nv[k]), spot_max[k], var_max)
           for k in range(len(K))]
    return ref, np.concatenate([r[0] for r in ref]), np.concatenate([r[1] for r in ref])


def test_batched_meshes_equal_per_option_meshes(golden):
    """heston_meshes_batch (lockstep bounded minimisation, native variance
    meshes) gives every option's meshes bit for bit, on the batched
    workload's box, the reference fixtures' cases and odd sizes."""
    rng = np.random.default_rng(11)
    n = 300
    K = 100 * rng.uniform(0.7, 1.3, n)
    v0 = rng.uniform(0.01, 0.16, n)
    nS = rng.choice(np.arange(64, 513, 32), n)
    nv = rng.choice(np.arange(32, 257, 16), n)
    K = np.concatenate([K, [100.0, 80.0, 100.0, 120.0, 93.0, 93.0]])
    v0 = np.concatenate([v0, [0.04] * 4, [0.07, 0.07]])
    nS = np.concatenate([nS, [150, 1024, 1024, 1024, 33, 3]])
    nv = np.concatenate([nv, [150, 512, 512, 512, 16, 8]])
    ref, S_ref, v_ref = _concat_ref(100.0, K, v0, nS, nv, 8.0 * K, 5.0)
    S, v = M.heston_meshes_batch(100.0, K, v0, nS, nv, 8.0 * K, 5.0)
    np.testing.assert_array_equal(S, S_ref)
    np.testing.assert_array_equal(v, v_ref)
    g = golden("meshes")
    so = np.concatenate([[0], np.cumsum(nS)])
    vo = np.concatenate([[0], np.cumsum(nv)])
    k = n  # the 150x150 configuration
    _same_as_fixture(S[so[k]:so[k + 1]], g["cfg1_S"])
    _same_as_fixture(v[vo[k]:vo[k + 1]], g["cfg1_v"])
    # the arena index of every price, by the same rounded bisection
    idx = M.price_index_batch(S, v, nS, nv, 100.0, v0)
    for k in range(len(K)):
        i, j = M.price_index(ref[k][0], ref[k][1], 100.0, v0[k])
        assert idx[k] == i * nv[k] + j


def test_batched_meshes_other_spot_and_range():
    """Spots off the strike grid, a wider spot range and the reference
    engine's defaults (S_max 1500, v_max 10)."""
    rng = np.random.default_rng(12)
    n = 64
    spot = rng.uniform(60, 140, n)
    K = rng.uniform(50, 150, n)
    v0 = rng.uniform(0.005, 0.3, n)
    nS = rng.integers(8, 300, n)
    nv = rng.integers(8, 200, n)
    for spot_max, var_max in ((8.0 * K, 5.0), (np.full(n, 1500.0), 10.0)):
        ref = [M.heston_meshes(spot[k], K[k], v0[k], int(nS[k]), int(nv[k]), spot_max[k], var_max)
               for k in range(n)]
        S, v = M.heston_meshes_batch(spot, K, v0, nS, nv, spot_max, var_max)
        np.testing.assert_array_equal(S, np.concatenate([r[0] for r in ref]))
        np.testing.assert_array_equal(v, np.concatenate([r[1] for r in ref]))


def test_native_exponential_space():
    """The library's host exponential_space against the Python restatement,
    bit for bit, and the reference's error when no point lies below v0."""
    import ctypes
    from fd_adi_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(13)
    for _ in range(400):
        v0 = rng.uniform(0.001, 0.3)
        n = int(rng.integers(2, 600))
        vmax = float(rng.choice([2.0, 5.0, 10.0]))
        ex = float(rng.choice([4.0, 3.0, 2.0, 1.0 / 3]))
        out = np.zeros(n)
        try:
            ref = M.exponential_space(0.0, v0, vmax, ex, n)
        except ValueError:
            assert lib.fdadi_exponential_space(0.0, v0, vmax, ex, n, 1, out.ctypes.data) == 1
            continue
        assert lib.fdadi_exponential_space(0.0, v0, vmax, ex, n, 1, out.ctypes.data) == 0
        np.testing.assert_array_equal(out, ref)
    out = np.zeros(4)
    assert lib.fdadi_exponential_space(0.0, 1e-6, 5.0, 4.0, 4, 1, out.ctypes.data) == 1
    assert "Did not find suitable value" in _lib.last_error()
    nv = np.array([4], dtype=np.int32)
    v0 = np.array([1e-6])
    rc = lib.fdadi_heston_var_meshes(1, v0.ctypes.data, nv.ctypes.data, 5.0, 4.0, 1, 0,
                                     out.ctypes.data)
    assert rc == 1 and "Did not find suitable value" in _lib.last_error()
