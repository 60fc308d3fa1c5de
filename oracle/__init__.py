"""CPU oracle of the D2Q9 hot path -- TEST INFRASTRUCTURE ONLY.

``d2q9`` is a numpy restatement of the reference's arithmetic (pinned
bit-exactly to the reference's own outputs by tests/golden), ``port`` a
ctypes binding of the multi-threaded C port in ``d2q9_port.c``.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py``
use this package, as the checker or as the timed CPU baseline; the product
(``latticeboltzmann_gb300``) never imports it.
"""
