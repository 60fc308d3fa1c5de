"""In-place streams (lbgb_stream_periodic_inplace, lbgb_stream_bounce_back_inplace)
against the out-of-place kernels, bit for bit.

The in-place path saves the edge values of every tile before any tile is
overwritten and streams each tile through shared memory; the cases cover
lattices smaller than one tile (16 rows x 512 bytes of a row), exactly one
tile, ragged tiles in both directions, rows that do not hold whole 16-byte
vectors and a population pointer that is not 16-byte aligned (scalar loads),
in every storage, periodic and with the cavity's walls and lid.  Lattices
whose rows hold whole 16-byte vectors take the pipelined kernel (one
persistent block per SM, two shared-memory stages, runs of four tiles along
y streamed in order with the column halo carried between them); the cases
cover runs of one to four tiles, a single run wrapping onto itself, ragged
last tiles in a run, and (the two largest) blocks that loop over several
runs.
"""

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from latticeboltzmann_gb300 import _lib

pytestmark = pytest.mark.gpu

STORAGES = {"f32": (_lib.F32, torch.float32), "f64": (_lib.F64, torch.float64),
            "f16dev": (_lib.F16DEV, torch.float16), "bf16dev": (_lib.BF16DEV, torch.bfloat16),
            "f32dev": (_lib.F32DEV, torch.float32)}
INT_VIEW = {2: torch.int16, 4: torch.int32, 8: torch.int64}
SIZES = [(1, 1), (2, 2), (3, 8), (2, 16), (17, 40), (16, 128), (16, 256), (33, 129), (50, 300), (64, 1032),
         (47, 2050), (300, 70), (700, 1024), (1000, 520)]


def raw_state(storage, nx, ny, seed, cuda, offset=0):
    """Stored values of a random near-equilibrium lattice (populations or
    scaled deviations), some of them signed zeros, in a buffer starting
    ``offset`` elements into its allocation."""
    g = torch.Generator().manual_seed(seed)
    h = 0.01 * torch.randn((9, nx, ny), generator=g, dtype=torch.float64)
    h[:, ::5, ::3] = -0.0
    if storage in ("f32", "f64"):
        w = torch.tensor([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=torch.float64)[:, None, None]
        vals = h + w
    elif storage == "f16dev":
        vals = h * 16384.0
    else:
        vals = h
    dt = STORAGES[storage][1]
    buf = torch.zeros(9 * nx * ny + offset, dtype=dt, device=cuda)
    view = buf[offset:].view(9, nx, ny)
    view.copy_(vals.to(dt))
    return buf, view


def run_inplace(view, nx, ny, code, boundary, u0):
    nbytes = int(_lib.load().lbgb_stream_inplace_workspace_bytes(nx, ny, code))
    ws = torch.empty(nbytes, dtype=torch.uint8, device=view.device)
    if boundary == "periodic":
        _lib.call("lbgb_stream_periodic_inplace", view.data_ptr(), nx, ny, code, ws.data_ptr(), nbytes, None)
    else:
        _lib.call("lbgb_stream_bounce_back_inplace", view.data_ptr(), nx, ny, u0, code, ws.data_ptr(), nbytes,
                  None)


def run_out_of_place(view, nx, ny, code, boundary, u0):
    out = torch.empty_like(view)
    if boundary == "periodic":
        _lib.call("lbgb_stream_periodic", view.data_ptr(), out.data_ptr(), nx, ny, code, None)
    else:
        _lib.call("lbgb_stream_bounce_back", view.data_ptr(), out.data_ptr(), nx, ny, u0, code, None)
    return out


@pytest.mark.parametrize("storage", list(STORAGES))
@pytest.mark.parametrize("boundary", ["periodic", "cavity"])
@pytest.mark.parametrize("nx,ny", SIZES)
def test_inplace_equals_out_of_place(cuda, storage, boundary, nx, ny):
    if boundary == "cavity" and (nx < 2 or ny < 2):
        pytest.skip("the cavity needs nx, ny >= 2")
    code, dt = STORAGES[storage]
    _, ref = raw_state(storage, nx, ny, nx * 131 + ny, cuda)
    _, g = raw_state(storage, nx, ny, nx * 131 + ny, cuda)
    for _ in range(3):
        ref = run_out_of_place(ref, nx, ny, code, boundary, 0.08)
        run_inplace(g, nx, ny, code, boundary, 0.08)
    torch.cuda.synchronize()
    iv = INT_VIEW[g.element_size()]
    assert torch.equal(g.view(iv), ref.view(iv))


@pytest.mark.parametrize("storage", ["f32", "f16dev", "f64"])
@pytest.mark.parametrize("boundary", ["periodic", "cavity"])
def test_inplace_unaligned_pointer(cuda, storage, boundary):
    """A population pointer one element past a 16-byte boundary takes the
    scalar load path; the result is the same."""
    nx, ny = 37, 520
    code, _ = STORAGES[storage]
    _, ref = raw_state(storage, nx, ny, 5, cuda)
    buf, g = raw_state(storage, nx, ny, 5, cuda, offset=1)
    assert g.data_ptr() % 16 != 0
    ref = run_out_of_place(ref, nx, ny, code, boundary, 0.1)
    run_inplace(g, nx, ny, code, boundary, 0.1)
    torch.cuda.synchronize()
    iv = INT_VIEW[g.element_size()]
    assert torch.equal(g.view(iv), ref.view(iv))
    assert float(buf[0]) == 0.0  # the element before the lattice is untouched


def test_inplace_operators_match_oracle_loop(cuda):
    """PyLB.Streaming on FP64 in place against the oracle's streams."""
    from oracle import d2q9 as oracle
    rng = np.random.default_rng(3)
    nx, ny = 70, 300
    f0 = oracle.equilibrium(1 + 0.02 * rng.standard_normal((nx, ny)), 0.03 * rng.standard_normal((nx, ny)),
                            0.03 * rng.standard_normal((nx, ny)))
    g = torch.from_numpy(f0).to(cuda)
    ref = f0.copy()
    for _ in range(4):
        PyLB.Streaming.stream_and_bounce_back(g, 0.1)
        oracle.stream_and_bounce_back(ref, 0.1)
        PyLB.stream(g)
        oracle.stream(ref)
    assert np.abs(g.cpu().numpy() - ref).max() <= 1e-15


def test_inplace_workspace_checked(cuda):
    nx, ny = 40, 256
    f = torch.zeros((9, nx, ny), dtype=torch.float32, device=cuda)
    need = int(_lib.load().lbgb_stream_inplace_workspace_bytes(nx, ny, _lib.F32))
    ws = torch.empty(need + 16, dtype=torch.uint8, device=cuda)
    with pytest.raises(ValueError, match="workspace"):
        _lib.call("lbgb_stream_periodic_inplace", f.data_ptr(), nx, ny, _lib.F32, ws.data_ptr(), need - 1, None)
    with pytest.raises(ValueError, match="16-byte"):
        _lib.call("lbgb_stream_bounce_back_inplace", f.data_ptr(), nx, ny, 0.1, _lib.F32, ws.data_ptr() + 4,
                  need, None)
    with pytest.raises(ValueError, match="cavity"):
        _lib.call("lbgb_stream_bounce_back_inplace", f.data_ptr(), 1, ny, 0.1, _lib.F32, ws.data_ptr(), need,
                  None)
