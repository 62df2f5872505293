"""chemsim_gb300 — GB300-native (sm_103a) D2Q9 lattice-Boltzmann step.

A drop-in for taktoa/chemsim's src/lbm.rs lattice storage and State::step:
the product is the C-ABI library liblbm_cuda.so (include/lbm_cuda.h) built
from csrc/; `lbm` mirrors lbm.rs's API over it.
"""
from .build import build  # noqa: F401
