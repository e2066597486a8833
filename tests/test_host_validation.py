"""Host-side validation of the C ABI: every entry point checks shapes,
pointers and plans before touching a device, and reports the reference's
error texts ("Vector too short to use finite differencing.", "Dimension
mismatch", "Vector length does not divide"; BandedOperator.pyx:43,
_TriBandedOperatorGPU.cu:1039). Runs without a GPU: no call here reaches a
kernel."""
import ctypes

import numpy as np
import pytest

from fd_adi_gb300 import _lib

FAKE = 0x1000   # a non-null pointer that is never dereferenced on these paths


def _batch(n0, n1, scheme=_lib.SCHEME_HV, n_steps=3, plan=None):
    n0 = np.asarray(n0, np.int32)
    n1 = np.asarray(n1, np.int32)
    b = _lib.HestonBatch(len(n0), scheme, n_steps, 2, 0.6, 0.5, 0, 0,
                         n0.ctypes.data, n1.ctypes.data, FAKE, FAKE, FAKE, FAKE, None,
                         ctypes.cast(ctypes.pointer(plan), ctypes.c_void_p) if plan else None)
    return b, (n0, n1, plan)   # keep the arrays alive with the struct


def test_short_lines_are_rejected():
    lib = _lib.load()
    b, keep = _batch([32, 3], [16, 16])
    assert lib.fdadi_heston_workspace_bytes(ctypes.byref(b)) == -1
    assert "Vector too short" in _lib.last_error()
    b, keep = _batch([32, 8], [16, 2])
    assert lib.fdadi_heston_workspace_bytes(ctypes.byref(b)) == -1
    assert "Vector too short" in _lib.last_error()


def test_scheme_and_step_counts_are_checked():
    lib = _lib.load()
    b, keep = _batch([32], [16], scheme=7)
    assert lib.fdadi_heston_workspace_bytes(ctypes.byref(b)) == -1
    assert "scheme" in _lib.last_error()
    b, keep = _batch([32], [16], n_steps=-1)
    assert lib.fdadi_heston_workspace_bytes(ctypes.byref(b)) == -1


@pytest.mark.parametrize("scheme", [_lib.SCHEME_DOUGLAS, _lib.SCHEME_HV, _lib.SCHEME_CS,
                                    _lib.SCHEME_MCS])
def test_workspace_grows_with_the_batch(scheme):
    lib = _lib.load()
    b1, k1 = _batch([32], [16], scheme=scheme)
    b2, k2 = _batch([32, 64, 5], [16, 40, 4], scheme=scheme)
    w1 = lib.fdadi_heston_workspace_bytes(ctypes.byref(b1))
    w2 = lib.fdadi_heston_workspace_bytes(ctypes.byref(b2))
    assert 0 < w1 < w2
    # a predictor/corrector scheme keeps F(V), Y2 and the corrector copies
    bd, kd = _batch([32], [16], scheme=_lib.SCHEME_DOUGLAS)
    if scheme != _lib.SCHEME_DOUGLAS:
        assert w1 > lib.fdadi_heston_workspace_bytes(ctypes.byref(bd))


def test_too_small_workspace_is_rejected():
    lib = _lib.load()
    b, keep = _batch([32], [16])
    need = lib.fdadi_heston_workspace_bytes(ctypes.byref(b))
    rc = lib.fdadi_heston_prepare(ctypes.byref(b), ctypes.c_void_p(FAKE), need - 256, None)
    assert rc == 3 and "workspace too small" in _lib.last_error()


def test_unknown_plans_are_rejected_before_any_launch():
    lib = _lib.load()
    plan = _lib.HestonPlan.from_dict({"spot_kind": 1, "spot_a": 7, "spot_b": 3,
                                      "var_kind": 0, "var_warps": 4})
    b, keep = _batch([32], [16], plan=plan)
    need = lib.fdadi_heston_workspace_bytes(ctypes.byref(b))
    rc = lib.fdadi_heston_run(ctypes.byref(b), ctypes.c_void_p(FAKE), need, ctypes.c_void_p(FAKE),
                              None)
    assert rc == 1 and "spot-solve plan" in _lib.last_error()
    plan = _lib.HestonPlan.from_dict({"spot_kind": 0, "spot_a": 1, "spot_b": 128,
                                      "var_kind": 3, "var_warps": 5})
    b, keep = _batch([32], [16], plan=plan)
    rc = lib.fdadi_heston_run(ctypes.byref(b), ctypes.c_void_p(FAKE), need, ctypes.c_void_p(FAKE),
                              None)
    assert rc == 1 and "variance-solve plan" in _lib.last_error()
    plan = _lib.HestonPlan.from_dict({"spot_kind": 0, "spot_a": 1, "spot_b": 128,
                                      "var_kind": 0, "var_warps": 4, "groups": 9})
    b, keep = _batch([32], [16], plan=plan)
    rc = lib.fdadi_heston_run(ctypes.byref(b), ctypes.c_void_p(FAKE), need, ctypes.c_void_p(FAKE),
                              None)
    assert rc == 1 and "groups" in _lib.last_error()


def test_default_plan_follows_the_batch_size():
    lib = _lib.load()
    small, k1 = _batch([64] * 4, [32] * 4)
    big, k2 = _batch([64] * 5000, [32] * 5000)
    p1, p2 = _lib.HestonPlan(), _lib.HestonPlan()
    assert lib.fdadi_heston_default_plan(ctypes.byref(small), ctypes.byref(p1)) == 0
    assert lib.fdadi_heston_default_plan(ctypes.byref(big), ctypes.byref(p2)) == 0
    assert p1.spot_a == 8 and p2.spot_a == 1        # few lines: prefetching loop


def test_tridiagonal_shape_errors():
    lib = _lib.load()
    f = [FAKE] * 8
    t = _lib.Tri(96, 32, 0, 0, 0, 0, 0, 0, *f)                 # 3 rows per block
    assert lib.fdadi_tri_apply(ctypes.byref(t), FAKE, FAKE, 3, 32, None) == 1
    assert "Vector too short" in _lib.last_error()
    t = _lib.Tri(128, 32, 0, 0, 0, 0, 0, 0, *f)
    assert lib.fdadi_tri_solve(ctypes.byref(t), FAKE, 8, 16, FAKE, None) == 1
    assert "Dimension mismatch" in _lib.last_error()
    t = _lib.Tri(130, 32, 0, 0, 0, 0, 0, 0, *f)
    assert lib.fdadi_tri_apply(ctypes.byref(t), FAKE, FAKE, 10, 13, None) == 1
    assert "does not divide" in _lib.last_error()


def test_no_alloc_solve_limit():
    lib = _lib.load()
    f = [FAKE] * 8
    rows = (1 << 20) + 64
    t = _lib.Tri(rows, 64, 1, 0, 0, 0, 0, 0, *f)
    assert lib.fdadi_tri_solve_noalloc(ctypes.byref(t), FAKE, 64, rows // 64, None) == 1
    assert "exceed" in _lib.last_error()


def test_gemm_and_inference_shape_errors():
    lib = _lib.load()
    g = _lib.Gemm(FAKE, 16, 0, FAKE, 16, 0, None, 0, None, 0, 0, FAKE, 16, 0, None, 0, 0,
                  100, 16, 16, 0, 1, 0, None)                 # M not a multiple of 128
    assert lib.fdadi_mlp_gemm(ctypes.byref(g), None) == 1
    assert "multiple of 128" in _lib.last_error()
    g = _lib.Gemm(FAKE, 24, 0, FAKE, 24, 0, None, 0, None, 0, 0, FAKE, 16, 0, None, 0, 0,
                  128, 16, 24, 0, 1, 0, None)                 # K not a multiple of 16
    assert lib.fdadi_mlp_gemm(ctypes.byref(g), None) == 1
    g = _lib.Gemm(FAKE, 16, 0, FAKE, 16, 0, None, 0, None, 0, 0, FAKE, 16, 0, None, 0, 0,
                  128, 16, 16, 0, 1, 5, None)                 # unknown variant
    assert lib.fdadi_mlp_gemm(ctypes.byref(g), None) == 1
    assert "variant" in _lib.last_error()
    net = _lib.MlpNet()
    for l, (k, n) in enumerate([(16, 256), (256, 256), (256, 256), (256, 256), (256, 128)]):
        net.W[l] = FAKE
        net.b[l] = FAKE
        net.K[l] = k
        net.N[l] = n
    net.members = 4
    net.N[2] = 192                                              # hidden width must be 256
    assert lib.fdadi_mlp_infer(ctypes.byref(net), FAKE, 256, FAKE, None, None) == 1
    assert "width" in _lib.last_error()
    net.N[2] = 256
    assert lib.fdadi_mlp_infer(ctypes.byref(net), FAKE, 200, FAKE, None, None) == 1
    assert "multiple of 128" in _lib.last_error()


def test_payoff_and_featurize_arguments():
    lib = _lib.load()
    b, keep = _batch([32, 40], [16, 20])
    need = lib.fdadi_heston_workspace_bytes(ctypes.byref(b))
    rc = lib.fdadi_heston_payoff(ctypes.byref(b), ctypes.c_void_p(FAKE), need, None, 0,
                                 ctypes.c_void_p(FAKE), None)
    assert rc == 1 and "null payoff argument" in _lib.last_error()
    rc = lib.fdadi_heston_payoff(ctypes.byref(b), ctypes.c_void_p(FAKE), need - 256,
                                 ctypes.c_void_p(FAKE), 0, ctypes.c_void_p(FAKE), None)
    assert rc == 3 and "workspace too small" in _lib.last_error()
    rc = lib.fdadi_mlp_featurize(FAKE, 128, FAKE, FAKE, 5, FAKE, FAKE, FAKE, None)
    assert rc == 1 and "control variate" in _lib.last_error()


def _bs(n, scheme=_lib.SCHEME_HV, n_steps=3, implicit=2):
    n = np.asarray(n, np.int32)
    return _lib.BsBatch(len(n), scheme, n_steps, implicit, 0.6, 0.5, n.ctypes.data, FAKE, FAKE,
                        FAKE, 0, 0), n


def test_black_scholes_batch_is_validated():
    """fdadi_bs_*: lines shorter than 4 points, unknown schemes and negative
    step counts are refused; the workspace holds 16 interleaved arrays padded
    to each warp group's longest line (groups of 32, longest lines first)."""
    lib = _lib.load()
    b, keep = _bs([64, 3])
    assert lib.fdadi_bs_workspace_bytes(ctypes.byref(b)) == -1
    assert "4 spot points" in _lib.last_error()
    b, keep = _bs([64], scheme=9)
    assert lib.fdadi_bs_workspace_bytes(ctypes.byref(b)) == -1
    assert "scheme" in _lib.last_error()
    b, keep = _bs([64], n_steps=-1)
    assert lib.fdadi_bs_workspace_bytes(ctypes.byref(b)) == -1
    sizes = np.random.default_rng(0).integers(4, 300, 100)
    b, keep = _bs(sizes)
    got = lib.fdadi_bs_workspace_bytes(ctypes.byref(b))
    srt = np.sort(sizes)[::-1]
    ni = sum(32 * int(srt[g * 32]) for g in range((len(srt) + 31) // 32))
    assert got >= 16 * 8 * ni
    assert got < 16 * 8 * ni + 8 * 4096   # the per-slot tables are small
    # the argument checks of the other entry points come before any launch
    assert lib.fdadi_bs_prepare(ctypes.byref(b), None, got, None) != 0
    assert lib.fdadi_bs_run(ctypes.byref(b), FAKE, got - 1, FAKE, None) == 3
    b.prefetch = 3
    assert lib.fdadi_bs_run(ctypes.byref(b), FAKE, got, FAKE, None) == 1
    assert "prefetch" in _lib.last_error()
