"""CPU oracle for the CUNFFT method (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline /
reference leg may use this package, and only as the checker or the timed CPU
baseline.  The GPU library never imports it.
"""
from .oracle import *  # noqa: F401,F403
