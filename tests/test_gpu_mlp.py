"""Tensor-core MLP kernels of the surrogate against torch on the same bf16
inputs (fp32 reference; tolerance 1e-4 relative to the result's scale, which
covers fp32 accumulation-order differences on K <= 512)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fd_adi_gb300 import _lib
    return _lib


def _gemm(L, A, B, M, N, K, problems=1, sA=0, sB=0, bias=None, sBias=0, aux=None, act=0,
          out_f32=None, out_bf16=None, status=None, variant=0, wait_cycles=0):
    g = L.Gemm(A.data_ptr(), A.shape[-1], sA, B.data_ptr(), B.shape[-1], sB,
               bias.data_ptr() if bias is not None else None, sBias,
               aux.data_ptr() if aux is not None else None, N, M * N,
               out_f32.data_ptr() if out_f32 is not None else None, N, M * N,
               out_bf16.data_ptr() if out_bf16 is not None else None, N, M * N,
               M, N, K, act, problems, variant,
               status.data_ptr() if status is not None else None, wait_cycles)
    L.call("fdadi_mlp_gemm", ctypes.byref(g),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


VARIANTS = [0, 1]   # 0: warp-specialised persistent TMA kernel; 1: two-stage cp.async kernel


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("M,N,K", [(128, 256, 256), (256, 16, 16), (384, 128, 96),
                                   (128, 32, 512)])
def test_umma_gemm_matches_torch(lib, M, N, K, variant):
    gen = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = torch.randn(M, K, generator=gen).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=gen).to(torch.bfloat16).cuda()
    C = torch.empty(M, N, dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _gemm(lib, A, B, M, N, K, out_f32=C, status=st, variant=variant)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.float() @ B.float().T
    assert (C - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()


@pytest.mark.parametrize("variant", VARIANTS)
def test_umma_gemm_epilogues_and_problems(lib, variant):
    M, N, K, P = 256, 256, 128, 3
    gen = torch.Generator(device="cpu").manual_seed(5)
    A = torch.randn(M, K, generator=gen).to(torch.bfloat16).cuda()          # shared input
    B = (torch.randn(P, N, K, generator=gen) * 0.1).to(torch.bfloat16).cuda()
    bias = torch.randn(P, N, generator=gen).cuda()
    Y = torch.empty(P, M, N, dtype=torch.float32, device="cuda")
    H = torch.empty(P, M, N, dtype=torch.bfloat16, device="cuda")
    _gemm(lib, A, B, M, N, K, problems=P, sA=0, sB=N * K, bias=bias, sBias=N, act=1,
          out_f32=Y, out_bf16=H, variant=variant)
    ref = torch.einsum("mk,pnk->pmn", A.float(), B.float()) + bias[:, None, :]
    torch.cuda.synchronize()
    assert (Y - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()
    href = torch.nn.functional.silu(ref)
    assert (H.float() - href).abs().max().item() <= 1e-2 * href.abs().max().item()
    # act 2: multiply by SiLU'(aux)
    aux = torch.randn(P, M, N, generator=gen).cuda()
    G = torch.empty(P, M, N, dtype=torch.bfloat16, device="cuda")
    _gemm(lib, A, B, M, N, K, problems=P, sA=0, sB=N * K, aux=aux, act=2, out_bf16=G,
          variant=variant)
    s = torch.sigmoid(aux)
    gref = torch.einsum("mk,pnk->pmn", A.float(), B.float()) * (s * (1 + aux * (1 - s)))
    torch.cuda.synchronize()
    assert (G.float() - gref).abs().max().item() <= 1e-2 * gref.abs().max().item()


def test_persistent_gemm_many_tiles(lib):
    """More 128-row tiles than SMs: every CTA loops over several units and
    reuses both tensor-memory accumulators."""
    M, N, K, P = 128 * 300, 256, 256, 2
    gen = torch.Generator(device="cpu").manual_seed(9)
    A = torch.randn(P, M, K, generator=gen).to(torch.bfloat16).cuda()
    B = (torch.randn(P, N, K, generator=gen) * 0.1).to(torch.bfloat16).cuda()
    bias = torch.randn(P, N, generator=gen).cuda()
    Y = torch.empty(P, M, N, dtype=torch.float32, device="cuda")
    H = torch.empty(P, M, N, dtype=torch.bfloat16, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _gemm(lib, A, B, M, N, K, problems=P, sA=M * K, sB=N * K, bias=bias, sBias=N, act=1,
          out_f32=Y, out_bf16=H, status=st)
    ref = torch.einsum("pmk,pnk->pmn", A.float(), B.float()) + bias[:, None, :]
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert (Y - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()
    href = torch.nn.functional.silu(ref)
    assert (H.float() - href).abs().max().item() <= 1e-2 * href.abs().max().item()


@pytest.mark.parametrize("N", [256, 16])
def test_split_k_weight_gradient_shape(lib, N):
    """Few output tiles and a long K (the weight-gradient GEMMs): K is split
    across CTAs and the fp32 partial sums are added atomically."""
    M, K, P = 256, 8192, 4
    gen = torch.Generator(device="cpu").manual_seed(N)
    A = torch.randn(P, M, K, generator=gen).to(torch.bfloat16).cuda()
    B = torch.randn(P, N, K, generator=gen).to(torch.bfloat16).cuda()
    C = torch.full((P, M, N), 7.0, dtype=torch.float32, device="cuda")   # overwritten
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _gemm(lib, A, B, M, N, K, problems=P, sA=M * K, sB=N * K, out_f32=C, status=st)
    ref = torch.einsum("pmk,pnk->pmn", A.float(), B.float())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert (C - ref).abs().max().item() <= 2e-4 * ref.abs().max().item()


def test_transpose_and_adam(lib):
    R, C = 300, 70
    x = torch.randn(R, C).to(torch.bfloat16).cuda()
    y = torch.empty(C, R, dtype=torch.bfloat16, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib.call("fdadi_transpose_bf16", ctypes.c_void_p(x.data_ptr()), C, 0,
             ctypes.c_void_p(y.data_ptr()), R, 0, R, C, 1, st)
    torch.cuda.synchronize()
    assert torch.equal(y, x.T)
    n, rows, cols = 64 * 48, 64, 48
    p = torch.randn(n, device="cuda")
    g = torch.randn(n, device="cuda")
    m1 = torch.zeros(n, device="cuda")
    m2 = torch.zeros(n, device="cuda")
    w = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    wt = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    p_ref = p.clone()
    lib.call("fdadi_mlp_adam", ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(g.data_ptr()),
             ctypes.c_void_p(m1.data_ptr()), ctypes.c_void_p(m2.data_ptr()), n, rows, cols,
             1e-3, 0.9, 0.999, 1e-8, 1, ctypes.c_void_p(w.data_ptr()),
             ctypes.c_void_p(wt.data_ptr()), st)
    torch.cuda.synchronize()
    # first Adam step: update = lr * g / (|g| + eps)
    ref = p_ref - 1e-3 * g / (g.abs() + 1e-8)
    assert (p - ref).abs().max().item() < 1e-6
    assert torch.equal(w, p.to(torch.bfloat16))
    assert torch.equal(wt.view(cols, rows), p.to(torch.bfloat16).view(rows, cols).T)


def test_bounded_wait_gives_up_and_context_stays_usable(lib):
    """The warp-specialised GEMM's abort path: its MMA warp waits on a barrier
    that nothing completes (wait_cycles < 0) until the limit (about 0.1 ms)
    runs out; the kernel must drain its copies and MMAs, free its tensor
    memory, set the status word and return. A normal launch afterwards on the
    same stream gives the right result, twice."""
    M, N, K = 256, 128, 256
    gen = torch.Generator(device="cpu").manual_seed(9)
    A = torch.randn(M, K, generator=gen).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=gen).to(torch.bfloat16).cuda()
    ref = A.float() @ B.float().T
    for _ in range(2):
        C = torch.zeros(M, N, dtype=torch.float32, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        _gemm(lib, A, B, M, N, K, out_f32=C, status=st, variant=0, wait_cycles=-200000)
        torch.cuda.synchronize()
        assert int(st.item()) == 1
        st.zero_()
        _gemm(lib, A, B, M, N, K, out_f32=C, status=st, variant=0)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        assert (C - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()
