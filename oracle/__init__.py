"""CPU oracle for the solve path — TEST INFRASTRUCTURE ONLY.

`femoracle` (oracle/*.c) restates the reference's routines in plain C; the
optional `ref` library (oracle/_ref, built from the reference's own sources
by oracle/Makefile) pins that restatement.  Only tests, the smoke entry
point and the CPU-baseline leg of bench.py import this package; the product
library never does.
"""
from .pyoracle import *  # noqa: F401,F403
