"""CPU oracle for the MORIS element hot path -- TEST INFRASTRUCTURE ONLY.

Imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` as the checker.  The product package ``moris_gb300`` never
imports it.  ``Oracle`` wraps ``fem_oracle.cpp`` through ctypes.
"""
from .oracle import OracleLib, OracleModel, load  # noqa: F401
