"""GB300-native HSS hot path with the HssMatrices.jl interface.

The package directory name contains a dot, so it is imported by path under the
module name ``hssmatrices_gb300`` (see ``__graft_entry__.load_package``).
"""
from .hssmatrix import (ClusterTree, HssMatrix, HssOptions, bisection_cluster, gensize, hssrank,
                        isbranch, isleaf, setopts)
from .linalg import DeviceHss, UlvFactor, ldiv, matmul, mul, ulvfactor, ulvfactsolve
from .packing import pack
from .synthetic import generator_entries, synthetic_hss
from . import _lib

__all__ = [
    "ClusterTree", "HssMatrix", "HssOptions", "bisection_cluster", "gensize", "hssrank", "isbranch",
    "isleaf", "setopts", "DeviceHss", "UlvFactor", "ldiv", "matmul", "mul", "ulvfactor",
    "ulvfactsolve", "pack", "synthetic_hss", "generator_entries",
]
