"""``PyLB.Streaming`` (PyLB/Streaming.py:28-46): ``c_ic`` and ``stream``, plus
the cavity walls ``stream_and_bounce_back``, ``bounce_back`` and
``moving_wall`` (cavity_opt1.py:177-245), from
``latticeboltzmann_gb300.Streaming``."""

from latticeboltzmann_gb300.Streaming import (__all__, bounce_back, c_ic, moving_wall, stream,  # noqa: F401
                                              stream_and_bounce_back)
