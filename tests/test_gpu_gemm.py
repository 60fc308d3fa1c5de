"""The BF16 GEMM (tensor-core tcgen05 path and CUDA-core reference) against a
float64 product of the same BF16-rounded operands."""

import numpy as np
import pytest
import torch

from latticeboltzmann_gb300 import _lib

pytestmark = pytest.mark.gpu


def gemm(A, B, C, alpha=1.0, beta=0.0, engine=0, batch=1, a_bs=0, b_bs=0, c_bs=0, dims=None):
    m, k = dims[0], dims[2]
    n = dims[1]
    _lib.call("lbgb_gemm_bf16", m, n, k, A.data_ptr(), A.stride(-2), A.stride(-1), a_bs, B.data_ptr(), B.stride(-2),
              B.stride(-1), b_bs, C.data_ptr(), C.stride(-2), C.stride(-1), c_bs, batch, alpha, beta,
              int(C.dtype == torch.bfloat16), engine, torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("m,n,k", [(128, 32, 64), (128, 64, 64), (256, 128, 128), (200, 48, 100), (1, 3, 5),
                                   (1000, 24, 256), (384, 96, 32), (130, 130, 70), (4096, 128, 32), (512, 3, 128),
                                   (512, 24, 24), (300, 64, 33), (2048, 32, 8), (256, 200, 16),
                                   (32, 32, 1600), (40, 4, 1000), (160, 32, 704)])
@pytest.mark.parametrize("layout", ["nn", "nt", "tn", "tt"])
@pytest.mark.parametrize("engine", [0, 1, 2])
def test_gemm_matches_float64(cuda, m, n, k, layout, engine):
    g = torch.Generator(device="cpu").manual_seed(m * 7 + n + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16)
    b = torch.randn(k, n, generator=g).to(torch.bfloat16)
    ref = a.double() @ b.double()
    A = (a if layout[0] == "n" else a.t().contiguous().t()).to(cuda)
    B = (b if layout[1] == "n" else b.t().contiguous().t()).to(cuda)
    C = torch.full((m, n), 7.0, device=cuda)
    gemm(A, B, C, dims=(m, n, k), engine=engine)
    _lib.call("lbgb_gemm_status", 1)
    err = (C.double().cpu() - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()), err
    # beta accumulates into C
    gemm(A, B, C, alpha=0.5, beta=1.0, dims=(m, n, k), engine=engine)
    err = (C.double().cpu() - 1.5 * ref).abs().max().item()
    assert err <= 2e-4 * max(1.0, ref.abs().max().item()), err


def test_gemm_batched_strides(cuda):
    z, m, n, k = 5, 96, 40, 72
    g = torch.Generator(device="cpu").manual_seed(3)
    a = torch.randn(z, m, k, generator=g).to(torch.bfloat16)
    b = torch.randn(z, k, n, generator=g).to(torch.bfloat16)
    ref = torch.bmm(a.double(), b.double())
    A, B = a.to(cuda), b.to(cuda)
    for engine in (1, 2):
        C = torch.zeros(z, m, n, device=cuda)
        gemm(A, B, C, engine=engine, batch=z, a_bs=m * k, b_bs=k * n, c_bs=m * n, dims=(m, n, k))
        assert (C.double().cpu() - ref).abs().max().item() < 1e-4 * ref.abs().max().item()
    _lib.call("lbgb_gemm_status", 1)


@pytest.mark.parametrize("engine", [1, 2])
def test_gemm_bf16_output_and_offsets(cuda, engine):
    """BF16 output is the FP32 result rounded once; unaligned operand starts
    (odd element offsets) take the scalar load path and stay exact."""
    m, n, k = 300, 40, 136
    g = torch.Generator(device="cpu").manual_seed(9)
    a = torch.randn(m, k + 1, generator=g).to(torch.bfloat16).to(cuda)[:, 1:]
    b = torch.randn(k, n, generator=g).to(torch.bfloat16).to(cuda)
    ref = a.double() @ b.double()
    C32 = torch.empty(m, n, device=cuda)
    gemm(a, b, C32, dims=(m, n, k), engine=engine)
    C16 = torch.empty(m, n, device=cuda, dtype=torch.bfloat16)
    gemm(a, b, C16, dims=(m, n, k), engine=engine)
    _lib.call("lbgb_gemm_status", 1)
    assert (C32.double() - ref).abs().max().item() < 1e-4 * ref.abs().max().item()
    assert torch.equal(C16, C32.to(torch.bfloat16))


@pytest.mark.parametrize("engine", [0, 1])
def test_gemm_empty_inner_dimension(cuda, engine):
    """K = 0: C = beta C (no tensor-core work is issued)."""
    A = torch.zeros(64, 0, dtype=torch.bfloat16, device=cuda)
    B = torch.zeros(0, 32, dtype=torch.bfloat16, device=cuda)
    C = torch.full((64, 32), 3.0, device=cuda)
    _lib.call("lbgb_gemm_bf16", 64, 32, 0, A.data_ptr(), 1, 1, 0, B.data_ptr(), 32, 1, 0, C.data_ptr(), 32, 1, 0, 1,
              1.0, 0.5, 0, engine, torch.cuda.current_stream().cuda_stream)
    _lib.call("lbgb_gemm_status", 1)
    assert torch.all(C == 1.5)


def _call(m, n, k, A, a, B, b, C, c, batch, alpha, beta, engine):
    _lib.call("lbgb_gemm_bf16", m, n, k, A.data_ptr(), a[0], a[1], a[2], B.data_ptr(), b[0], b[1], b[2], C.data_ptr(),
              c[0], c[1], c[2], batch, alpha, beta, int(C.dtype == torch.bfloat16), engine,
              torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("m,n,k,batch,shared_b", [(128, 32, 64, 1, False), (1000, 24, 256, 1, False),
                                                  (130, 130, 72, 1, False), (4096, 128, 24, 1, False),
                                                  (300, 64, 40, 3, False), (256, 48, 256, 4, True),
                                                  (33, 7, 8, 1, False), (640, 256, 24, 2, True),
                                                  (129, 96, 1032, 2, False)])
@pytest.mark.parametrize("out", ["f32_rows", "f32_cols", "bf16_rows"])
@pytest.mark.parametrize("a_major", ["k", "m"])
def test_tma_pipeline_k_major(cuda, m, n, k, batch, shared_b, out, a_major):
    """The TMA + warp-specialised tcgen05 kernel (engine 3: B K-major, A
    K-major or M-major): ragged M, N and K tails, batched problems with their
    own or a shared B, FP32 output in either layout and BF16 output, alpha
    and beta, against a float64 product of the same BF16 operands."""
    g = torch.Generator(device="cpu").manual_seed(m + 3 * n + 7 * k + batch)
    a = torch.randn(batch, m, k, generator=g).to(torch.bfloat16)
    bt = torch.randn(1 if shared_b else batch, n, k, generator=g).to(torch.bfloat16)  # B(k, n) = bt[n, k]
    ref = torch.einsum("zmk,znk->zmn", a.double(), bt.double().expand(batch, n, k))
    A, Bt = a.to(cuda), bt.to(cuda)
    dt = torch.bfloat16 if out == "bf16_rows" else torch.float32
    if out == "f32_cols":
        Cs = torch.full((batch, n, m), 2.0, device=cuda)
        C, c = Cs, (1, m, m * n)
    else:
        C = torch.full((batch, m, n), 2.0, device=cuda, dtype=dt)
        c = (n, 1, m * n)
    if a_major == "k":
        _call(m, n, k, A, (k, 1, m * k), Bt, (1, k, 0 if shared_b else n * k), C, c, batch, 0.5, 0.25, 3)
    else:
        if m % 8:
            pytest.skip("M-major rows need m a multiple of 8 (16-byte aligned)")
        At = a.transpose(1, 2).contiguous().to(cuda)  # (batch, k, m): A(m, k) = At[k, m]
        _call(m, n, k, At, (1, m, m * k), Bt, (1, k, 0 if shared_b else n * k), C, c, batch, 0.5, 0.25, 3)
    _lib.call("lbgb_gemm_status", 1)
    got = C.double().cpu()
    if out == "f32_cols":
        got = got.transpose(1, 2)
    want = 0.5 * ref + 0.25 * 2.0
    tol = (1e-2 if dt == torch.bfloat16 else 1e-4) * max(1.0, want.abs().max().item())
    assert (got - want).abs().max().item() <= tol


def test_tma_pipeline_split_k_strides(cuda):
    """The weight-gradient pattern: one long K split into batched chunks whose
    batch stride (the chunk) is smaller than the row stride (all of K)."""
    M, N, K, S = 32, 32, 8192, 8
    ks = K // S
    g = torch.Generator(device="cpu").manual_seed(11)
    a = torch.randn(M, K, generator=g).to(torch.bfloat16)
    bt = torch.randn(N, K, generator=g).to(torch.bfloat16)
    parts = torch.zeros(S, M, N, device=cuda)
    _call(M, N, ks, a.to(cuda), (K, 1, ks), bt.to(cuda), (1, K, ks), parts, (N, 1, M * N), S, 1.0, 0.0, 0)
    _lib.call("lbgb_gemm_status", 1)
    ref = torch.stack([a[:, i * ks:(i + 1) * ks].double() @ bt[:, i * ks:(i + 1) * ks].double().t()
                       for i in range(S)])
    assert (parts.double().cpu() - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()


def test_tma_engine_rejects_other_layouts(cuda):
    A = torch.zeros(64, 16, dtype=torch.bfloat16, device=cuda)
    B = torch.zeros(16, 32, dtype=torch.bfloat16, device=cuda)
    C = torch.zeros(64, 32, device=cuda)
    with pytest.raises(ValueError):  # B is N-major here
        _call(64, 32, 16, A, (16, 1, 0), B, (32, 1, 0), C, (32, 1, 0), 1, 1.0, 0.0, 3)


@pytest.mark.parametrize("rows_per_bias", [4096, 300, 16])
@pytest.mark.parametrize("act", [0, 1])
def test_gemm_bias_act_equals_gemm_then_bias_act(cuda, rows_per_bias, act):
    """The TMA pipeline's fused bias + activation epilogue (one Fourier layer:
    C = A B + C, C += bias per channel block of rows, BF16 copy of GELU(C))
    gives the values of lbgb_gemm_bf16 followed by lbgb_fno_bias_act: C bit
    for bit, the BF16 copy within one BF16 rounding step."""
    m, n, k = 4096, 64, 24
    g = torch.Generator(device="cpu").manual_seed(rows_per_bias + act)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16).to(cuda)                   # K-major A
    bt = torch.randn(n, k, generator=g).to(torch.bfloat16).to(cuda)                  # B^T stored: K-major B
    c0 = torch.randn(m, n, generator=g).to(cuda)
    nb = (m + rows_per_bias - 1) // rows_per_bias
    bias = torch.randn(nb, generator=g).to(cuda)
    s = torch.cuda.current_stream().cuda_stream
    # unfused: GEMM with beta = 1, then the bias pass per row block (channels x cols)
    c1 = c0.clone()
    _lib.call("lbgb_gemm_bf16", m, n, k, a.data_ptr(), k, 1, 0, bt.data_ptr(), 1, k, 0, c1.data_ptr(), n, 1, 0, 1,
              1.0, 1.0, 0, 3, s)
    vb1 = torch.empty(m, n, dtype=torch.bfloat16, device=cuda)
    if m % rows_per_bias == 0:
        _lib.call("lbgb_fno_bias_act", c1.data_ptr(), bias.data_ptr(), None, None, vb1.data_ptr(), nb,
                  rows_per_bias * n, act, s)
    else:
        # ragged last block: the bias pass row block by row block
        for i in range(nb):
            r0, r1 = i * rows_per_bias, min(m, (i + 1) * rows_per_bias)
            _lib.call("lbgb_fno_bias_act", c1[r0:r1].data_ptr(), bias[i:].data_ptr(), None, None,
                      vb1[r0:r1].data_ptr(), 1, (r1 - r0) * n, act, s)
    c2 = c0.clone()
    vb2 = torch.empty(m, n, dtype=torch.bfloat16, device=cuda)
    _lib.call("lbgb_gemm_bf16_bias_act", m, n, k, a.data_ptr(), k, 1, bt.data_ptr(), k, c2.data_ptr(), n, 1.0, 1.0,
              bias.data_ptr(), rows_per_bias, act, vb2.data_ptr(), s)
    _lib.call("lbgb_gemm_status", 1)
    assert torch.equal(c1, c2)
    d = (vb1.float() - vb2.float()).abs()
    assert (d <= 2 ** -7 * vb1.float().abs().clamp_min(2 ** -100)).all()


def test_gemm_bias_act_rejects_other_layouts(cuda):
    m, n, k = 256, 32, 16
    a = torch.zeros(k, m, dtype=torch.bfloat16, device=cuda)  # M-major A
    bt = torch.zeros(n, k, dtype=torch.bfloat16, device=cuda)
    c = torch.zeros(m, n, device=cuda)
    rc = _lib.load().lbgb_gemm_bf16_bias_act(m, n, k, a.data_ptr(), 1, m, bt.data_ptr(), k, c.data_ptr(), n, 1.0, 0.0,
                                             None, 1, 0, None, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.EUNSUPPORTED
