"""TEST INFRASTRUCTURE ONLY: Python access to the CPU checkers.

``port`` wraps liboracle.so, the plain-C restatement of the reference solver (lbm_oracle.c);
``ref`` wraps oracle/_ref/libref_lbm.so, the reference's own headers compiled by oracle/Makefile
(present only where the reference tree was available at build time). Only tests/,
__graft_entry__.smoke() and bench.py's CPU arm may use this package; the product library never
does.
"""
from .checkers import Checker, build, port_available, ref_available, run_port, run_ref

__all__ = ["Checker", "build", "port_available", "ref_available", "run_port", "run_ref"]
