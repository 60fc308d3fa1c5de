"""Argument checks shared by the operator modules.

The reference binds its kernels through pybind11 with non-const
``Eigen::Ref`` arguments (c/_lbkernels.cpp:33-49): an array of the wrong dtype
or layout matches no overload and raises ``TypeError``, and the call mutates
the caller's buffer in place.  The checks below keep that contract for CUDA
tensors: wrong type, device, dtype or layout -> ``TypeError``; wrong shape ->
``ValueError``.  Host arrays are rejected: there is no CPU path.
"""

import torch

from . import _lib

_DTYPES = {torch.float32: _lib.F32, torch.float64: _lib.F64}


def require_cuda(t, name):
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s: expected a CUDA torch.Tensor, got %s (there is no CPU path)" % (name, type(t).__name__))
    if t.device.type != "cuda":
        raise TypeError("%s: expected a CUDA tensor, got one on %s (there is no CPU path)" % (name, t.device))
    return t


def storage_code(t, name):
    try:
        return _DTYPES[t.dtype]
    except KeyError:
        raise TypeError("%s: dtype %s not supported (float32 or float64)" % (name, t.dtype)) from None


def stream_handle(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def population_view(f, name):
    """Checks a (9, N) or (9, nx, ny) population tensor; returns (n, chan_stride).

    Channels may be spaced by any stride >= N; the cells of one channel must be
    contiguous (the layout the reference's Eigen::Ref<Array<T,9,Dynamic,RowMajor>>
    accepts).
    """
    require_cuda(f, name)
    if f.dim() not in (2, 3) or f.shape[0] != 9:
        raise ValueError("%s: expected shape (9, N) or (9, nx, ny), got %s" % (name, tuple(f.shape)))
    if f.dim() == 2:
        n = f.shape[1]
        if n > 1 and f.stride(1) != 1:
            raise TypeError("%s: cells of a channel must be contiguous" % name)
    else:
        n = f.shape[1] * f.shape[2]
        if n > 0 and not f[0].is_contiguous():
            raise TypeError("%s: cells of a channel must be contiguous" % name)
    cs = f.stride(0) if n > 0 else 0
    if n > 0 and cs < n:
        raise TypeError("%s: channel stride %d is smaller than the %d cells of a channel" % (name, cs, n))
    return n, max(cs, n)


def lattice(f, name):
    """Checks a C-contiguous (9, nx, ny) population tensor; returns (nx, ny)."""
    require_cuda(f, name)
    if f.dim() != 3 or f.shape[0] != 9:
        raise ValueError("%s: expected shape (9, nx, ny), got %s" % (name, tuple(f.shape)))
    if not f.is_contiguous():
        raise TypeError("%s: population tensor must be C-contiguous" % name)
    return f.shape[1], f.shape[2]
