"""BGK collision and equilibrium on the GPU (drop-in for PyLB.Collision).

The reference module is a pass-through to its native extension
(PyLB/Collision.py:21 -> c/_lbkernels.cpp:33-49 -> c/d2q9.h).  Here the same
two calls launch sm_103a kernels of liblbgb on CUDA tensors, on the current
torch stream, and mutate the caller's tensor in place.
"""

import torch

from . import _lib
from ._tensor import population_view, require_cuda, storage_code, stream_handle

__all__ = ["collide", "equilibrium"]


def collide(f, omega, keep_mass=False):
    """Relax populations towards equilibrium, in place (c/d2q9.h:121-131).

    Parameters
    ----------
    f : torch.Tensor
        CUDA tensor of shape ``(9, N)`` (or ``(9, nx, ny)``), float32 or float64;
        channel rows may be spaced by any stride, cells of a channel contiguous.
        Modified in place.
    omega : float
        Relaxation parameter.
    keep_mass : bool
        False (default): the native kernel's arithmetic operation by
        operation, so the result equals ``d2q9_colliden`` bit for bit in
        float32 and float64.  True: the fused solver's collision, whose
        float32 store writes the rest population last so that each node keeps
        its mass up to one rounding (no counterpart in the reference).

    Returns None, like the reference binding.
    """
    n, cs = population_view(f, "collide")
    code = storage_code(f, "collide")
    if n == 0:
        return None
    flags = _lib.COLLIDE_KEEP_MASS if keep_mass else 0
    _lib.call("lbgb_collide_ex", f.data_ptr(), n, cs, code, float(omega), flags, stream_handle(f))
    return None


def _scalar_equilibrium(rho, ux, uy):
    # The reference registers the float overload first (c/_lbkernels.cpp:36), so
    # Python scalars give a float32 (9,) vector; 0-d tensors keep their dtype.
    dev = None
    dtype = torch.float32
    for v in (rho, ux, uy):
        if isinstance(v, torch.Tensor):
            require_cuda(v, "equilibrium")
            dev, dtype = v.device, v.dtype
    if dev is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    vals = [v.reshape(1).to(dtype) if isinstance(v, torch.Tensor) else torch.tensor([float(v)], dtype=dtype, device=dev)
            for v in (rho, ux, uy)]
    f = torch.empty((9, 1), dtype=dtype, device=dev)
    code = storage_code(f, "equilibrium")
    _lib.call("lbgb_equilibrium", vals[0].data_ptr(), vals[1].data_ptr(), vals[2].data_ptr(), f.data_ptr(), 1, 1,
              code, stream_handle(f))
    return f.reshape(9)


def equilibrium(rho, ux, uy, f=None):
    """Equilibrium populations (c/d2q9.h:59-81 and :98-108).

    ``equilibrium(rho, ux, uy)`` with scalars returns a ``(9,)`` CUDA tensor.
    ``equilibrium(rho, ux, uy, f)`` with fields of N cells writes the
    equilibrium into ``f`` (shape ``(9, N)``) in place and returns None.
    """
    if f is None:
        if all(not isinstance(v, torch.Tensor) or v.dim() == 0 for v in (rho, ux, uy)):
            return _scalar_equilibrium(rho, ux, uy)
        raise TypeError("equilibrium: field arguments need an output array f of shape (9, N)")
    n, cs = population_view(f, "equilibrium")
    code = storage_code(f, "equilibrium")
    fields = []
    for name, v in (("rho", rho), ("ux", ux), ("uy", uy)):
        require_cuda(v, "equilibrium")
        if v.dtype != f.dtype:
            raise TypeError("equilibrium: %s has dtype %s, f has %s" % (name, v.dtype, f.dtype))
        if v.numel() < n:
            raise ValueError("equilibrium: %s has %d values, f has %d cells" % (name, v.numel(), n))
        if not v.is_contiguous():
            raise TypeError("equilibrium: %s must be contiguous" % name)
        if v.device != f.device:
            raise TypeError("equilibrium: %s is on %s, f on %s" % (name, v.device, f.device))
        fields.append(v)
    if n == 0:
        return None
    _lib.call("lbgb_equilibrium", fields[0].data_ptr(), fields[1].data_ptr(), fields[2].data_ptr(), f.data_ptr(), n,
              cs, code, stream_handle(f))
    return None
