"""Host mesh generators against the reference's meshes."""
import numpy as np

from fd_adi_gb300 import mesh as M


def test_heston_meshes(golden):
    g = golden("meshes")
    S, v = M.heston_meshes(100., 100., 0.04, 150, 150, 800., 5.)
    np.testing.assert_array_equal(S, g["cfg1_S"])
    np.testing.assert_array_equal(v, g["cfg1_v"])
    S, v = M.heston_meshes(100., 100., 0.04, 150, 150, 1500., 10.)
    np.testing.assert_array_equal(S, g["def_S"])
    np.testing.assert_array_equal(v, g["def_v"])
    for K in (80, 100, 120):
        S, v = M.heston_meshes(100., float(K), 0.04, 1024, 512, 8.0 * K, 5.)
        np.testing.assert_array_equal(S, g["cfg2_S_K%d" % K])
        np.testing.assert_array_equal(v, g["cfg2_v_K%d" % K])
    for n in (33, 64, 96, 150, 256, 512):
        S, v = M.heston_meshes(100., 93., 0.07, n, max(8, n // 2), 8 * 93., 5.)
        np.testing.assert_array_equal(S, g["var_S_%d" % n])
        np.testing.assert_array_equal(v, g["var_v_%d" % n])


def test_bs_and_barrier_meshes(golden):
    g = golden("meshes")
    np.testing.assert_array_equal(M.sinh_space(100., 5000., 1.0, 150), g["bs_S"])
    np.testing.assert_array_equal(M.barrier_spots(100., 170., 60), g["barrier_S"])


def test_price_index():
    S = np.array([0.0, 50.0, 99.99999, 100.0, 150.0])
    assert M.price_index(S, np.array([0.0, 0.04, 1.0]), 100.0, 0.04) == (2, 1)
