"""GB300-native D2Q9 lattice-Boltzmann hot path behind the PyLB operator API.

``import latticeboltzmann_gb300 as PyLB`` gives the reference package's
surface (PyLB/__init__.py:21-22): ``collide``, ``equilibrium`` and ``stream``
at the top level, and the ``Collision``, ``Streaming`` and ``IO`` modules.
Every operator takes CUDA tensors and runs hand-written sm_103a kernels from
liblbgb.so; there is no CPU path.  ``Lattice`` is the device-resident solver
(fused stream + collide, ping-pong buffers, CUDA-graph capture).
"""

from . import Collision, IO, Streaming
from .Collision import collide, equilibrium
from .Streaming import stream
from .solver import Lattice, fft_amplitude, macroscopic, mass_momentum, omega_from_reynolds, viscosity_from_omega

__all__ = ["collide", "equilibrium", "stream", "Collision", "Streaming", "IO", "Lattice", "macroscopic",
           "mass_momentum", "omega_from_reynolds", "viscosity_from_omega"]
