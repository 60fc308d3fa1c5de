"""``PyLB.IO`` (PyLB/IO.py:27-80): ``save_mpiio`` (single rank) and
``save_npy`` from ``latticeboltzmann_gb300.IO``."""

from latticeboltzmann_gb300.IO import __all__, npy_header, save_mpiio, save_npy  # noqa: F401
