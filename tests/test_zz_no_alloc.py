"""fdadi_tri_solve_noalloc: the tridiagonal solve for callers that cannot
allocate device memory (their host owns every byte of it, or they run a
latency-critical loop where cudaMalloc/cudaFree would synchronize the
device). It must give what fdadi_tri_solve gives with caller scratch, call
after call, since every call reuses the library's one static scratch array.
This file is collected last so a stop-at-first-failure run has already run
everything else."""
import ctypes

import numpy as np
import pytest

from fd_adi_gb300 import _lib


def _operators():
    from fd_adi_gb300.construct import make_operators
    from fd_adi_gb300.engine import heston_coefficients, heston_boundaries
    from fd_adi_gb300 import mesh
    S, v = mesh.heston_meshes(100., 100., 0.04, 150, 150, 800., 5.)
    ops = make_operators([S, v], heston_coefficients(0.06, 1.0, 0.04, 0.5, -0.7),
                         heston_boundaries())
    A0, A1 = ops[0].to_gpu(), ops[1].to_gpu()
    # the implicit-stage operators 1 - theta*dt*A of a Douglas step
    Li0 = A0 * (0.5 * -1.0 / 150)
    Li0.add(1, inplace=True)
    Li1 = A1 * (0.5 * -1.0 / 150)
    Li1.add(1, inplace=True)      # CAN_FOLD: the solve folds the corner on the fly
    Li1f = Li1.copy()
    Li1f.diagonalize()            # FOLDED
    return S.size, v.size, [Li0, Li1, Li1f]


@pytest.mark.gpu
def test_noalloc_solve_matches_scratch_solve_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    n0, n1, ops = _operators()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    scratch = torch.empty(n0 * n1, dtype=torch.float64, device="cuda")
    gen = torch.Generator(device="cpu").manual_seed(11)
    for op in ops:
        tri = op._tri()
        for call in range(2):   # two calls in a row, different right-hand sides
            X = (torch.rand(n0, n1, generator=gen, dtype=torch.float64) * 600).cuda()
            ref = X.clone()
            rc = lib.fdadi_tri_solve(ctypes.byref(tri), ctypes.c_void_p(ref.data_ptr()), n0, n1,
                                     ctypes.c_void_p(scratch.data_ptr()), st)
            _lib.check(rc, "fdadi_tri_solve")
            got = X.clone()
            rc = lib.fdadi_tri_solve_noalloc(ctypes.byref(tri), ctypes.c_void_p(got.data_ptr()),
                                             n0, n1, st)
            _lib.check(rc, "fdadi_tri_solve_noalloc")
            torch.cuda.synchronize()
            r, g = ref.cpu().numpy(), got.cpu().numpy()
            assert np.abs(g - r).max() <= 1e-13 * np.abs(r).max(), (op.axis, call)


def test_noalloc_rejects_operators_beyond_its_scratch():
    """The size check happens on the host before any device work."""
    lib = _lib.load()
    n0, n1 = 2048, 1024            # 2^21 rows > FDADI_NOALLOC_MAX_ROWS
    dummy = 256                    # never dereferenced: the call returns first
    tri = _lib.Tri(n0 * n1, n1, 0, 0, 0, 0, 0, 0, dummy, dummy, dummy, dummy, dummy, dummy,
                   dummy, dummy)
    rc = lib.fdadi_tri_solve_noalloc(ctypes.byref(tri), ctypes.c_void_p(dummy), n0, n1, None)
    assert rc == 1
    msg = _lib.last_error()
    assert "exceed" in msg and str(_lib.NOALLOC_MAX_ROWS) in msg
