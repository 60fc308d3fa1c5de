"""The reference's package name, ``PyLB``, over the GB300 solver.

The reference's drivers and tests import the operators as ``import PyLB as
D2Q9`` and ``from PyLB.IO import save_mpiio``
(simulators/parallel_lid_drive_cavity/cavity_opt2.py:42-43,
tests/01-ImportTest.py:43-44); the package re-exports the operator surface of
PyLB/__init__.py:21-22 from ``latticeboltzmann_gb300``, whose calls run the
sm_103a kernels of liblbgb.so on CUDA tensors.  The submodules ``Collision``,
``Streaming`` and ``IO`` re-export those of ``latticeboltzmann_gb300`` under
the reference's names.
"""

from . import IO, Collision, Streaming  # noqa: F401
from .Collision import collide, equilibrium  # noqa: F401
from .Streaming import stream  # noqa: F401

__all__ = ["collide", "equilibrium", "stream", "Collision", "Streaming", "IO"]
