"""GB300-native Monte Carlo sweep for ETHER (mukkelian/Ether).

The compute path is libether_gpu.so (hand-written sm_103a CUDA behind the C-ABI in
include/ether_gpu.h); this package is its Python binding and host-side set-up helpers.
"""
from . import abi
from .abi import EtherError, MODEL_ISING, MODEL_XYZ, FLAG_FORCE_GENERAL, FLAG_NO_GRAPHS, \
    FLAG_NO_RESIDENT, FLAG_PT_REFERENCE_COPY, FLAG_PT_TRUE_ENERGY, FLAG_STAGED_SPINS
from .model import KB_EV, MB_EV, Batch, Lattice, Learned, Sweep, couplings, learn_batch_sweep, local_111_axes, \
    pyrochlore, run, simple_cubic, units

__all__ = ["abi", "EtherError", "MODEL_ISING", "MODEL_XYZ", "FLAG_FORCE_GENERAL",
           "FLAG_PT_REFERENCE_COPY", "FLAG_NO_GRAPHS", "FLAG_NO_RESIDENT", "FLAG_PT_TRUE_ENERGY",
           "FLAG_STAGED_SPINS", "KB_EV", "MB_EV", "Batch", "Lattice", "Learned",
           "Sweep", "couplings", "learn_batch_sweep", "local_111_axes", "pyrochlore", "run", "simple_cubic", "units"]
