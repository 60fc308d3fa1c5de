"""Streaming, bounce-back and moving wall on the GPU (drop-in for PyLB.Streaming).

``stream`` replaces PyLB/Streaming.py:33-46.  The reference keeps its wall
treatment in the cavity scripts (``stream_and_bounce_back``,
simulators/parallel_lid_drive_cavity/cavity_opt1.py:177-245); it is offered
here as part of the module, with the same semantics, plus ``bounce_back``
(resting walls) and ``moving_wall`` (an alias taking the lid velocity).

All calls act in place on a C-contiguous CUDA tensor of shape ``(9, nx, ny)``
through the library's in-place streams: the values that neighbouring tiles
pull across tile edges are saved into a small workspace (about 5 % of the
lattice, from torch's caching allocator), then every tile is streamed in
shared memory and written back over itself -- one read and one write of the
lattice plus the edges, with results equal to the out-of-place kernels' bit
for bit.  A time loop that owns its buffers should use
``latticeboltzmann_gb300.Lattice`` (fused stream + collide, 72 bytes per FP32
cell and step).
"""

import numpy as np
import torch

from . import _lib
from ._tensor import lattice, storage_code, stream_handle

__all__ = ["c_ic", "stream", "stream_and_bounce_back", "bounce_back", "moving_wall"]

# "Velocities" of the channels, x and y components (PyLB/Streaming.py:28-29).
c_ic = np.array([[0, 1, 0, -1, 0, 1, -1, -1, 1],
                 [0, 0, 1, 0, -1, 1, 1, -1, -1]]).T


def _workspace(f_ikl, nx, ny, code):
    """Edge-record workspace of one in-place stream, from torch's caching
    allocator on the tensor's device (stream-ordered: reused only after the
    call that held it)."""
    nbytes = int(_lib.load().lbgb_stream_inplace_workspace_bytes(nx, ny, code))
    return torch.empty(max(nbytes, 16), dtype=torch.uint8, device=f_ikl.device), nbytes


def stream(f_ikl):
    """Propagate every channel by one cell with periodic wrap, in place.

    ``f_i(k, l) <- f_i((k - c_ix) mod nx, (l - c_iy) mod ny)``.
    """
    nx, ny = lattice(f_ikl, "stream")
    code = storage_code(f_ikl, "stream")
    if f_ikl.numel() == 0:
        return None
    ws, nbytes = _workspace(f_ikl, nx, ny, code)
    _lib.call("lbgb_stream_periodic_inplace", f_ikl.data_ptr(), nx, ny, code, ws.data_ptr(), nbytes,
              stream_handle(f_ikl))
    return None


def stream_and_bounce_back(f_ikl, u0=0.1):
    """Stream with half-way bounce-back on all four walls and a lid moving with ``u0``.

    Every node is a fluid node; the walls sit half a cell outside the array.
    The lid is the wall at ``l = ny - 1`` and moves in +x; populations leaving
    through it get the Ladd term ``+-6 w_i rho_lid u0``.  Semantics, including
    the reference's corner order and lid density, are those of
    cavity_opt1.py:177-245.  Needs ``nx >= 2`` and ``ny >= 2``.
    """
    nx, ny = lattice(f_ikl, "stream_and_bounce_back")
    code = storage_code(f_ikl, "stream_and_bounce_back")
    if nx < 2 or ny < 2:
        raise ValueError("stream_and_bounce_back: the cavity needs nx >= 2 and ny >= 2, got %d x %d" % (nx, ny))
    ws, nbytes = _workspace(f_ikl, nx, ny, code)
    _lib.call("lbgb_stream_bounce_back_inplace", f_ikl.data_ptr(), nx, ny, float(u0), code, ws.data_ptr(),
              nbytes, stream_handle(f_ikl))
    return None


def bounce_back(f_ikl):
    """Stream with resting no-slip walls on all four sides (``u0 = 0``), in place."""
    return stream_and_bounce_back(f_ikl, 0.0)


def moving_wall(f_ikl, u0):
    """Stream with bounce-back and the top wall moving with velocity ``u0`` in +x."""
    return stream_and_bounce_back(f_ikl, u0)
