"""Field output in the .npy format (drop-in for PyLB.IO).

The reference writes a global 2-D field collectively with MPI-IO
(PyLB/IO.py:27-80): a version-1.0 header whose dictionary is padded with
spaces so that magic + length + dictionary end on a 16-byte boundary,
followed by the C-ordered data.  On one GPU there is one writer: the field
is copied device -> host once (pinned staging) and written with that same
header layout, so files are byte-identical to the reference's at one rank
and load with ``numpy.load``.
"""

import struct

import numpy as np
import torch

__all__ = ["save_mpiio", "save_npy", "npy_header"]

_MAGIC = b"\x93NUMPY\x01\x00"


def npy_header(dtype, shape):
    """Header bytes of a version-1.0 .npy file, padded as PyLB/IO.py:55-61 pads it."""
    descr = np.lib.format.dtype_to_descr(np.dtype(dtype))
    d = str({"descr": descr, "fortran_order": False, "shape": tuple(int(s) for s in shape)})
    # dictionary + magic(8) + length(2) must be 15 mod 16 before the newline
    while (len(d) + len(_MAGIC) + 2) % 16 != 15:
        d += " "
    d += "\n"
    return _MAGIC + struct.pack("<H", len(d)) + d.encode("latin-1")


def _host(g):
    if isinstance(g, torch.Tensor):
        if g.device.type == "cuda":
            h = torch.empty(g.shape, dtype=g.dtype, pin_memory=True)
            h.copy_(g)
            return h.numpy()
        return g.numpy()
    return np.asarray(g)


def save_npy(fn, g_kl):
    """Write a 2-D field (CUDA tensor or array) to ``fn`` in .npy format."""
    a = np.ascontiguousarray(_host(g_kl))
    if a.ndim != 2:
        raise ValueError("save_npy: expected a 2-D field, got shape %s" % (a.shape,))
    with open(fn, "wb") as fh:
        fh.write(npy_header(a.dtype, a.shape))
        fh.write(a.tobytes(order="C"))


def save_mpiio(comm, fn, g_kl):
    """Signature of PyLB.IO.save_mpiio (PyLB/IO.py:27).

    ``comm`` may be None or any communicator of size 1 (``Get_size()``); with
    one GPU per process the whole field lives in this process.  A larger
    communicator is rejected: the distributed writer is outside this library.
    """
    if comm is not None and hasattr(comm, "Get_size") and comm.Get_size() != 1:
        raise NotImplementedError("save_mpiio: only a single-rank communicator is supported")
    save_npy(fn, g_kl)
