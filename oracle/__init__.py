"""The oracle: a CPU restatement of taktoa/chemsim's D2Q9 step (src/lbm.rs).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs, as the checker and the timed CPU baseline; the shipped
library (chemsim_gb300) never imports it.  Parity against the reference is
unpinned (the reference cannot run here); see lbm_oracle.cpp's header.
"""
from .oracle import (  # noqa: F401
    build, lib_path, step, equilibrium, moments, health, max_threads,
)
