"""The allocation-free reduction entry point, called through the C ABI.

Callers that may not allocate device memory (a code embedded in an
application whose memory manager owns the GPU, or a time loop that forbids
device allocations between steps) cannot hand lbgb_mass_momentum a workspace;
lbgb_mass_momentum_noalloc keeps its partial sums in an array built into the
library instead.  This file is collected last on purpose: it exercises the
library-wide array after everything else has run, and also passes on its own
in a fresh process.
"""

import ctypes

import numpy as np
import pytest
import torch

from latticeboltzmann_gb300 import _lib

pytestmark = pytest.mark.gpu

CODES = {torch.float32: _lib.F32, torch.float64: _lib.F64}


def with_workspace(lib, f, n, cs, code, stream):
    out = torch.empty(3, dtype=torch.float64, device=f.device)
    nbytes = lib.lbgb_mass_momentum_workspace_bytes()
    ws = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=f.device)
    rc = lib.lbgb_mass_momentum(f.data_ptr(), n, cs, code, out.data_ptr(), ws.data_ptr(), ws.numel() * 8, stream)
    assert rc == _lib.OK, _lib.last_error()
    return out


def test_no_alloc_reduction_matches_workspace_reduction(cuda):
    lib = _lib.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    rng = np.random.default_rng(2024)
    # two calls in a row on different lattices: the second must not see the
    # first call's partial sums left in the shared array
    cases = [((9, 300, 257), torch.float64), ((9, 64, 4096), torch.float32)]
    for shape, dtype in cases:
        f = torch.from_numpy(0.02 + 0.2 * rng.random(shape)).to(dtype=dtype, device=cuda)
        n = shape[1] * shape[2]
        ref = with_workspace(lib, f, n, n, CODES[dtype], stream)
        out = torch.full((3,), float("nan"), dtype=torch.float64, device=cuda)
        rc = lib.lbgb_mass_momentum_noalloc(f.data_ptr(), n, n, CODES[dtype], out.data_ptr(), stream)
        assert rc == _lib.OK, _lib.last_error()
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        # same tolerance as the workspace reduction's own test against the oracle
        assert np.abs(a - b).max() < 1e-9, (a, b)
        # and both agree with a float64 sum on the host
        h = f.double().cpu().numpy()
        cx = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])[:, None, None]
        cy = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])[:, None, None]
        assert np.abs(a - [h.sum(), (cx * h).sum(), (cy * h).sum()]).max() < 1e-9


def test_no_alloc_reduction_rejects_oversized_lattices(cuda):
    lib = _lib.load()
    f = torch.zeros((9, 4), dtype=torch.float32, device=cuda)
    out = torch.zeros(3, dtype=torch.float64, device=cuda)
    too_many = _lib.NOALLOC_MAX_CELLS + 1
    # rejected on the host before any launch (the sizes are never dereferenced)
    rc = lib.lbgb_mass_momentum_noalloc(f.data_ptr(), too_many, too_many, _lib.F32, out.data_ptr(),
                                        ctypes.c_void_p(None))
    assert rc == _lib.EINVAL
    assert "scratch limit" in _lib.last_error()
