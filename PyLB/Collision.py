"""``PyLB.Collision`` (PyLB/Collision.py:21): ``collide`` and ``equilibrium``
of ``latticeboltzmann_gb300.Collision`` on CUDA tensors."""

from latticeboltzmann_gb300.Collision import __all__, collide, equilibrium  # noqa: F401
