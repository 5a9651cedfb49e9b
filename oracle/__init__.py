"""CPU oracle for the minimmerflow Euler step (test infrastructure only).

Only the test suite, the smoke check and the CPU-baseline leg of bench.py may
import this package.  It wraps ``mmf_oracle.c`` (a plain-C restatement of the
reference algorithm) through ctypes; see ``mmf_oracle.h`` for the citations.
"""
from .binding import *  # noqa: F401,F403
