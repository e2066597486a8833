"""Host operator construction (fd_adi_gb300.construct) against the reference's
own operators (tests/golden/operators.npz), bit for bit."""
import numpy as np

from fd_adi_gb300.construct import make_operators
from fd_adi_gb300.engine import heston_coefficients, heston_boundaries


def test_heston_operators_bitwise(golden):
    g = golden("operators")
    r, kappa, theta, sigma, rho = g["params"]
    ops = make_operators([g["S"], g["v"]], heston_coefficients(r, kappa, theta, sigma, rho),
                         heston_boundaries())
    np.testing.assert_array_equal(ops[0].rows, g["A0"])
    np.testing.assert_array_equal(ops[0].R, g["R0"])
    np.testing.assert_array_equal(ops[1].rows, g["A1"])
    np.testing.assert_array_equal(ops[1].R, g["R1"])
    assert ops[1].bot_status == "CAN_FOLD" and ops[0].bot_status == "CANNOT_FOLD"
    coeff, w0, w1, n0, n1 = ops[(0, 1)].mixed
    M = np.zeros((n0 * n1, n0 * n1))
    for i in range(1, n0 - 1):
        for j in range(1, n1 - 1):
            for a in (-1, 0, 1):
                for b in (-1, 0, 1):
                    M[i * n1 + j, (i + a) * n1 + j + b] = w1[b + 1][j] * w0[a + 1][i] * coeff[i * n1 + j]
    # the reference forms (w1*w0)*c; same products
    np.testing.assert_array_equal(M, g["M"])
