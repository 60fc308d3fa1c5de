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
@pytest.mark.parametrize("engine", [1, 2])
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
