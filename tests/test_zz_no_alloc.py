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

STORAGES = {"f32": (_lib.F32, torch.float32), "f64": (_lib.F64, torch.float64),
            "f16dev": (_lib.F16DEV, torch.int16), "bf16dev": (_lib.BF16DEV, torch.int16),
            "f32dev": (_lib.F32DEV, torch.float32)}


def with_workspace(lib, f, n, cs, code, stream):
    out = torch.empty(3, dtype=torch.float64, device=f.device)
    nbytes = lib.lbgb_mass_momentum_workspace_bytes()
    ws = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=f.device)
    rc = lib.lbgb_mass_momentum(f.data_ptr(), n, cs, code, out.data_ptr(), ws.data_ptr(), ws.numel() * 8, stream)
    assert rc == _lib.OK, _lib.last_error()
    return out


def stored(lib, pops, storage, stream):
    """The populations pops (float64, (9, nx, ny)) in the given storage."""
    code, dtype = STORAGES[storage]
    n = pops.shape[1] * pops.shape[2]
    f = torch.empty(pops.shape, dtype=dtype, device=pops.device)
    rc = lib.lbgb_convert(pops.data_ptr(), _lib.F64, n, f.data_ptr(), code, n, n, stream)
    assert rc == _lib.OK, _lib.last_error()
    return f


def decoded_sums(lib, f, storage, stream):
    """(mass, x momentum, y momentum) of the stored values, decoded to float64
    and summed on the host."""
    code, _ = STORAGES[storage]
    n = f.shape[1] * f.shape[2]
    h = torch.empty(f.shape, dtype=torch.float64, device=f.device)
    rc = lib.lbgb_convert(f.data_ptr(), code, n, h.data_ptr(), _lib.F64, n, n, stream)
    assert rc == _lib.OK, _lib.last_error()
    torch.cuda.synchronize()
    h = h.cpu().numpy()
    cx = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])[:, None, None]
    cy = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])[:, None, None]
    return np.array([h.sum(), (cx * h).sum(), (cy * h).sum()])


@pytest.mark.parametrize("storage", list(STORAGES))
def test_no_alloc_reduction_matches_workspace_reduction(cuda, storage):
    """Every storage code, on two calls in a row with different lattices:
    the second must not see the first call's partial sums left in the shared
    array.  The second lattice has more than 256 partials (9 x 1024 x 1100:
    275 blocks of 4096 cells), which the final pass sums in a strided loop."""
    lib = _lib.load()
    code, _ = STORAGES[storage]
    stream = torch.cuda.current_stream(cuda).cuda_stream
    rng = np.random.default_rng(2024)
    for shape in [(9, 300, 257), (9, 1024, 1100)]:
        pops = torch.from_numpy(0.02 + 0.2 * rng.random(shape)).to(cuda)
        f = stored(lib, pops, storage, stream)
        n = shape[1] * shape[2]
        ref = with_workspace(lib, f, n, n, code, stream)
        out = torch.full((3,), float("nan"), dtype=torch.float64, device=cuda)
        rc = lib.lbgb_mass_momentum_noalloc(f.data_ptr(), n, n, code, out.data_ptr(), stream)
        assert rc == _lib.OK, _lib.last_error()
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        # FP64 sums of ~1e5-1e6 values in two fixed orders
        tol = 1e-12 * np.abs(b).max() + 1e-9
        assert np.abs(a - b).max() < tol, (storage, a, b)
        # and both agree with a float64 sum of the decoded values on the host
        assert np.abs(a - decoded_sums(lib, f, storage, stream)).max() < tol, storage


def test_no_alloc_reduction_empty_lattice(cuda):
    """n = 0 after a call that filled the array: the sums are exactly zero."""
    lib = _lib.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    f = torch.full((9, 64, 64), 0.25, dtype=torch.float64, device=cuda)
    out = torch.empty(3, dtype=torch.float64, device=cuda)
    assert lib.lbgb_mass_momentum_noalloc(f.data_ptr(), 4096, 4096, _lib.F64, out.data_ptr(), stream) == _lib.OK
    out.fill_(float("nan"))
    rc = lib.lbgb_mass_momentum_noalloc(f.data_ptr(), 0, 0, _lib.F64, out.data_ptr(), stream)
    assert rc == _lib.OK, _lib.last_error()
    torch.cuda.synchronize()
    assert out.cpu().numpy().tolist() == [0.0, 0.0, 0.0]


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
