"""CPU oracle for the tracer path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this package.  The product (fv3atm_gb300) never loads it.
"""
from .oracle import *  # noqa: F401,F403
