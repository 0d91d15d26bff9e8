"""GB300-native Newman-Ziff bond percolation: a drop-in for the
``percolate.hpc`` path of andsor/pypercolate, computed by hand-written sm_103a
CUDA kernels in libnzgb300.so (C ABI: include/nz_gb300.h).

Modules
-------
hpc        drop-in of ``percolate.hpc`` (same functions, dtypes, errors)
percolate  ``spanning_2d_grid``, ``spanning_1d_chain``, ``percolation_graph``,
           ``_binomial_pmf``
ensemble   batched ensembles (many runs per launch, fused reductions)
"""
from . import hpc, percolate  # noqa: F401
from .percolate import (spanning_1d_chain, spanning_2d_grid,  # noqa: F401
                        percolation_graph)

__version__ = '0.1.0'
