"""GB300-native HSS hot path with the HssMatrices.jl interface.

The package directory name contains a dot, so it is imported by path under the
module name ``hssmatrices_gb300`` (see ``__graft_entry__.load_package``).
"""
from .hssmatrix import (ClusterTree, HssMatrix, HssOptions, bisection_cluster, gensize, hssrank,
                        isbranch, isleaf, setopts)
from .linalg import (DeviceHss, UlvFactor, cluster_trees, full, getindex, hss_ldiv, hssmul, ldiv, matmul, mul,
                     orthonormalize_generators, rdiv, recompress, rmatmul, transpose, ulvfactor, ulvfactsolve)
from .packing import pack, unpack
from .compression import (Compressor, DenseDevice, cluster_table, randcompress, randcompress_adaptive,
                          sample, sumsq)
from . import compression
from .synthetic import generator_entries, synthetic_hss
from . import _lib

__all__ = [
    "ClusterTree", "HssMatrix", "HssOptions", "bisection_cluster", "gensize", "hssrank", "isbranch",
    "isleaf", "setopts", "DeviceHss", "UlvFactor", "cluster_trees", "full", "getindex", "hss_ldiv", "hssmul",
    "ldiv", "orthonormalize_generators", "rdiv", "recompress", "rmatmul", "transpose", "matmul", "mul", "ulvfactor",
    "ulvfactsolve", "pack", "unpack", "synthetic_hss", "generator_entries", "Compressor", "DenseDevice",
    "cluster_table", "randcompress", "randcompress_adaptive", "sample", "sumsq", "compression",
]
